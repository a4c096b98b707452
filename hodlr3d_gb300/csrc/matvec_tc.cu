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
// Operands: every A row is a contiguous, 16-byte aligned run of FP32 values
// (rows of the row-major FP32 U, columns of the FP32 V, rows of the FP32
// near-field blocks), loaded with 128-bit loads; B is a [32][K] array.  The
// near-field blocks are the kernel evaluated once in FP32 with the same
// formula as the CUDA-core engine's on-the-fly near field.
//
// Products are split x = hi + lo into TF32 parts, A_hi B_hi + A_hi B_lo +
// A_lo B_hi (3xTF32).  The tensor core's FP32 accumulation is not rounded to
// nearest, so its error grows with the number of accumulations: each FP32
// accumulation group is kGroupChunks chunks (K <= 64) and groups are summed
// with compensated (Kahan) FP32 arithmetic, whose error matches an FP64 sum
// here at a fraction of the cost of GB300's FP64 units.  Two TMEM accumulators
// alternate between groups: one is read back while the next is multiplied.
//
// Per chunk (K = 32): wait until the operand stage (two alternate) is no
// longer read by the MMAs of two chunks ago, split and store the operands
// loaded into registers one chunk ahead, issue 12 MMAs from one thread,
// commit, load the next chunk.  Every mbarrier wait is bounded; a block whose
// wait gives up sets the error flag, drains with the same bound, frees TMEM.
#include <algorithm>

#include "matvec.h"
#include "tc.cuh"

namespace h3d {

namespace {

constexpr int NR = 32;                 // right-hand sides (MMA N)
constexpr int KC = 32;                 // K per chunk
constexpr int THREADS = 128;           // one row of the M = 128 tile per thread
constexpr int A_BYTES = 128 * KC * 4;  // one TF32 part of an A chunk (16 KB)
constexpr int B_BYTES = NR * KC * 4;   // one TF32 part of a B chunk (4 KB)
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int SMEM_BYTES = 2 * STAGE_BYTES;  // two operand stages
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t IDESC = tc::idesc_tf32(128, NR);
constexpr int kGroupChunks = 2;        // chunks per FP32 accumulation group (K <= 64)
constexpr int kMaxItems = 192;         // items (pairs, near blocks) of one block

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// One operand source of the long-K products: A element (row i, k) at
// a[i * as + k] for k < alen (alen a multiple of 4, zero padding), B element
// (c, k) at b[c * bs + k] for k < blen; blen is the item's K.
struct Item {
  const float* a;
  const float* b;
  int64_t as;
  int64_t bs;
  int alen;
  int blen;
};

struct Regs {
  float4 a[KC / 4];
  float b[8];
};

__device__ __forceinline__ void load_item(const Item& it, int k0, int row, bool live, Regs& R) {
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4* src = reinterpret_cast<const float4*>(it.a + (int64_t)row * it.as + k0);
#pragma unroll
  for (int q = 0; q < KC / 4; ++q) R.a[q] = (live && k0 + 4 * q < it.alen) ? src[q] : z;
  const int c = threadIdx.x & 31, kb = (threadIdx.x >> 5) * 8;
  const float* b = it.b + (int64_t)c * it.bs + k0 + kb;
#pragma unroll
  for (int j = 0; j < 8; ++j) R.b[j] = (k0 + kb + j < it.blen) ? b[j] : 0.f;
}

struct Stage {
  unsigned char* smem;
  __device__ __forceinline__ unsigned char* a_hi() const { return smem; }
  __device__ __forceinline__ unsigned char* a_lo() const { return smem + A_BYTES; }
  __device__ __forceinline__ unsigned char* b_hi() const { return smem + 2 * A_BYTES; }
  __device__ __forceinline__ unsigned char* b_lo() const { return smem + 2 * A_BYTES + B_BYTES; }
};

__device__ __forceinline__ void put4(unsigned char* hi, unsigned char* lo, uint32_t off, float4 x) {
  float4 h, l;
  tc::split_tf32(x.x, h.x, l.x);
  tc::split_tf32(x.y, h.y, l.y);
  tc::split_tf32(x.z, h.z, l.z);
  tc::split_tf32(x.w, h.w, l.w);
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

// a quarter-warp writes 8 consecutive rows of one k quad: no bank conflicts
__device__ __forceinline__ void store_regs(const Stage& S, const Regs& R) {
  const int row = threadIdx.x;
#pragma unroll
  for (int q = 0; q < KC / 4; ++q) put4(S.a_hi(), S.a_lo(), tc::kmajor_off(row, 4 * q, KC), R.a[q]);
  const int c = threadIdx.x & 31, kb = (threadIdx.x >> 5) * 8;
  put4(S.b_hi(), S.b_lo(), tc::kmajor_off(c, kb, KC), make_float4(R.b[0], R.b[1], R.b[2], R.b[3]));
  put4(S.b_hi(), S.b_lo(), tc::kmajor_off(c, kb + 4, KC), make_float4(R.b[4], R.b[5], R.b[6], R.b[7]));
}

// The block's tensor-core state: two operand stages, two accumulators.
struct Engine {
  Stage st[2];
  uint64_t* bar;      // bar[0..1]: operand stages, bar[2..3]: accumulators 0, 1
  uint32_t tmem;      // 64 columns: accumulator b at column 32 b
  int n_stage[2];
  int n_acc[2];
  int chunk;
  int* err;

  __device__ __forceinline__ void wait(int which, int n) {
    if (n > 0 && !tc::mbar_wait(&bar[which], (uint32_t)((n - 1) & 1), kWaitLimit)) atomicExch(err, 1);
  }
  __device__ __forceinline__ const Stage& next_stage() {
    const int s = chunk & 1;
    wait(s, n_stage[s]);
    return st[s];
  }
  __device__ __forceinline__ void issue(int buf, bool accumulate, bool close_group) {
    const int s = chunk & 1;
    tc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      const uint32_t d = tmem + 32u * (uint32_t)buf;
      const uint32_t ah = tc::smem_addr(st[s].a_hi()), al = tc::smem_addr(st[s].a_lo());
      const uint32_t bh = tc::smem_addr(st[s].b_hi()), bl = tc::smem_addr(st[s].b_lo());
#pragma unroll
      for (int ks = 0; ks < KC / 8; ++ks) {
        const uint32_t o = ks * 256;
        const uint64_t dah = tc::make_desc(ah + o, 128, KC * 32);
        const uint64_t dal = tc::make_desc(al + o, 128, KC * 32);
        const uint64_t dbh = tc::make_desc(bh + o, 128, KC * 32);
        const uint64_t dbl = tc::make_desc(bl + o, 128, KC * 32);
        tc::mma_tf32(d, dah, dbh, IDESC, (accumulate || ks > 0) ? 1u : 0u);
        tc::mma_tf32(d, dah, dbl, IDESC, 1u);
        tc::mma_tf32(d, dal, dbh, IDESC, 1u);
      }
      tc::mma_commit(&bar[s]);
      if (close_group) tc::mma_commit(&bar[2 + buf]);
    }
    ++n_stage[s];
    ++chunk;
    if (close_group) ++n_acc[buf];
  }
  __device__ __forceinline__ void read(int buf, float* v) {
    wait(2 + buf, n_acc[buf]);
    tc::fence_after_sync();
    tc::tmem_ld32(tmem + 32u * (uint32_t)buf + ((uint32_t)((threadIdx.x >> 5) * 32) << 16), v);
    tc::fence_before_sync();
    __syncthreads();
  }
};

__device__ __forceinline__ void engine_setup(Engine& E, unsigned char* smem, uint64_t* bar,
                                             uint32_t* tslot, int* err) {
  E.st[0].smem = smem;
  E.st[1].smem = smem + STAGE_BYTES;
  E.bar = bar;
  E.n_stage[0] = E.n_stage[1] = 0;
  E.n_acc[0] = E.n_acc[1] = 0;
  E.chunk = 0;
  E.err = err;
  if (threadIdx.x < 32) tc::tmem_alloc(tslot, 64);
  if (threadIdx.x == 0)
    for (int i = 0; i < 4; ++i) tc::mbar_init(&bar[i], 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  E.tmem = *tslot;
}

__device__ __forceinline__ void engine_teardown(Engine& E) {
  E.wait(0, E.n_stage[0]);
  E.wait(1, E.n_stage[1]);
  E.wait(2, E.n_acc[0]);
  E.wait(3, E.n_acc[1]);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(E.tmem, 64);
}

// Streams the items' chunks through the engine; the groups of kGroupChunks
// chunks are summed into (sum, comp) with compensated FP32 additions.
__device__ __forceinline__ void long_k(Engine& E, const Item* items, int nitems, bool live, float* sum,
                                   float* comp) {
  int it = 0;
  while (it < nitems && items[it].blen <= 0) ++it;
  if (it >= nitems) return;
  int k0 = 0, buf = 0, gchunks = 0;
  bool pending = false;
  Regs R;
  load_item(items[it], k0, threadIdx.x, live, R);
  for (;;) {
    int it2 = it, k2 = k0 + KC;
    if (k2 >= items[it].blen) {
      k2 = 0;
      ++it2;
      while (it2 < nitems && items[it2].blen <= 0) ++it2;
    }
    const bool has_next = it2 < nitems;
    const bool close = !has_next || gchunks + 1 == kGroupChunks;
    const Stage& S = E.next_stage();
    store_regs(S, R);
    E.issue(buf, gchunks > 0, close);
    ++gchunks;
    if (has_next) load_item(items[it2], k2, threadIdx.x, live, R);
    if (close) {
      if (pending) {
        float v[NR];
        E.read(buf ^ 1, v);
#pragma unroll
        for (int c = 0; c < NR; ++c) kahan_add(sum[c], comp[c], v[c]);
      }
      pending = true;
      buf ^= 1;
      gchunks = 0;
    }
    if (!has_next) break;
    it = it2;
    k0 = k2;
  }
  if (pending) {
    float v[NR];
    E.read(buf ^ 1, v);
#pragma unroll
    for (int c = 0; c < NR; ++c) kahan_add(sum[c], comp[c], v[c]);
  }
}

// ---------------------------------------------------------------------------
// Phase A: T = [F_p^T] X over one input box.  SLICE: the pairs of levels
// 1..d-1 over a level d-1 box; otherwise the leaf-level pairs over a leaf.
// Each block takes every gridDim.y-th tile of 128 concatenated pair columns.
template <bool SLICE>
__global__ void __launch_bounds__(THREADS) k_ta_tc(FarOp op, const float* __restrict__ Xt, int64_t N,
                                                   float* __restrict__ T, float* __restrict__ Pp,
                                                   int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[4];
  __shared__ uint32_t tslot;
  __shared__ int s_pair[kMaxItems];
  __shared__ int s_cum[kMaxItems + 1];
  Engine E;
  engine_setup(E, smem, bar, &tslot, err);
  const int d = op.levels;
  const int64_t box = blockIdx.x;
  const int sh_in = SLICE ? 3 : 0;
  const int64_t i0 = op.leaf_off[box << sh_in], i1 = op.leaf_off[(box + 1) << sh_in];
  const int kin = (int)(i1 - i0);
  const int jlo = SLICE ? 1 : d, jhi = SLICE ? d - 1 : d;
  for (int j = jlo; j <= jhi; ++j) {
    const int up = SLICE ? 3 * (d - 1 - j) : 0;
    const int64_t a = box >> up;
    const int64_t gb = level_base(j) + a;
    const int64_t a0 = op.leaf_off[a << (3 * (d - j))];
    const int64_t lda = op.leaf_off[(a + 1) << (3 * (d - j))] - a0;
    const int64_t mp = (lda + 3) & ~3;
    const int64_t ro = i0 - a0;
    const int slice_idx = (int)(box - (a << up));
    const bool to_t = !SLICE || j == d - 1;
    const int64_t q0 = op.il_ptr[gb], nq = op.il_ptr[gb + 1] - q0;
    for (int64_t qb = 0; qb < nq; qb += kMaxItems) {
      const int nb = (int)min((int64_t)kMaxItems, nq - qb);
      __syncthreads();
      if (threadIdx.x == 0) {
        int c = 0;
        for (int i = 0; i < nb; ++i) {
          const int p = op.rev[q0 + qb + i];
          s_pair[i] = p;
          s_cum[i] = c;
          c += op.rank[p];
        }
        s_cum[nb] = c;
      }
      __syncthreads();
      const int rows = s_cum[nb];
      const int ntiles = (rows + 127) / 128;
      for (int tile = blockIdx.y; tile < ntiles; tile += gridDim.y) {
        // this thread's pair column: A row = V_p column l over the input box
        const int rho = tile * 128 + (int)threadIdx.x;
        int p = -1, l = 0;
        if (rho < rows) {
          int lo = 0, hi = nb - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_cum[mid] <= rho) lo = mid;
            else hi = mid - 1;
          }
          p = s_pair[lo];
          l = rho - s_cum[lo];
        }
        Item it;
        it.a = p >= 0 ? static_cast<const float*>(op.vfac[p]) + (int64_t)l * mp + ro : Xt;
        it.as = 0;
        it.alen = kin;
        it.b = Xt + i0;
        it.bs = N;
        it.blen = kin;
        float sum[NR], comp[NR];
#pragma unroll
        for (int c = 0; c < NR; ++c) sum[c] = comp[c] = 0.f;
        long_k(E, &it, 1, p >= 0, sum, comp);
        if (p >= 0) {
          const int r = op.rank[p];
          float* dst = to_t ? T + op.tr_off[p] * NR
                            : Pp + (op.part_off[p] + (int64_t)slice_idx * r) * NR;
#pragma unroll
          for (int c = 0; c < NR; ++c) dst[(int64_t)c * r + l] = sum[c] - comp[c];
        }
      }
    }
  }
  engine_teardown(E);
}

// FP64 sum of slice partials: T_p[c][l] = sum_s P_p[s][c][l]
__global__ void k_tred_tc(FarOp op, const int32_t* __restrict__ pairs, const float* __restrict__ Pp,
                          float* __restrict__ T) {
  const int p = pairs[blockIdx.x];
  const int r = op.rank[p];
  const int64_t ns = int64_t(1) << (3 * (op.levels - 1 - op.pair_level[p]));
  const float* src = Pp + op.part_off[p] * NR;
  float* dst = T + op.tr_off[p] * NR;
  for (int o = threadIdx.x; o < r * NR; o += blockDim.x) {
    double acc = 0.0;
    for (int64_t s = 0; s < ns; ++s) acc += (double)src[s * r * NR + o];
    dst[o] = (float)acc;
  }
}

// Phase B over the levels above the leaves: one block per (slice, 128 rows).
__global__ void __launch_bounds__(THREADS) k_ut_tc(FarOp op, const float* __restrict__ T,
                                                   int64_t N, double* __restrict__ Ynl,
                                                   int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[4];
  __shared__ uint32_t tslot;
  __shared__ Item s_items[kMaxItems];
  Engine E;
  engine_setup(E, smem, bar, &tslot, err);
  const int d = op.levels;
  const int64_t sb = blockIdx.x;
  const int64_t s0 = op.leaf_off[sb << 3], s1 = op.leaf_off[(sb + 1) << 3];
  const int64_t r0 = s0 + 128 * (int64_t)blockIdx.y;
  const int nrows = (int)min((int64_t)128, s1 - r0);
  float sum[NR], comp[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) sum[c] = comp[c] = 0.f;
  if (nrows > 0) {
    for (int j = 1; j <= d - 1; ++j) {
      const int sh = 3 * (d - 1 - j);
      const int64_t a = sb >> sh;
      const int64_t gb = level_base(j) + a;
      const int64_t a0 = op.leaf_off[a << (sh + 3)];
      const int64_t q0 = op.il_ptr[gb], nq = op.il_ptr[gb + 1] - q0;
      for (int64_t qb = 0; qb < nq; qb += kMaxItems) {
        const int nb = (int)min((int64_t)kMaxItems, nq - qb);
        __syncthreads();
        for (int i = threadIdx.x; i < nb; i += THREADS) {
          const int p = (int)(q0 + qb + i);
          const int r = op.rank[p];
          const int rp = (r + 3) & ~3;
          Item it;
          it.a = static_cast<const float*>(op.ufac[p]) + (r0 - a0) * rp;
          it.as = rp;
          it.alen = rp;
          it.b = T + op.tr_off[p] * NR;
          it.bs = r;
          it.blen = r;
          s_items[i] = it;
        }
        __syncthreads();
        long_k(E, s_items, nb, (int)threadIdx.x < nrows, sum, comp);
      }
    }
  }
  const int row = threadIdx.x;
  if (row < nrows) {
#pragma unroll
    for (int c = 0; c < NR; ++c) Ynl[(int64_t)c * N + r0 + row] = (double)sum[c] - (double)comp[c];
  }
  engine_teardown(E);
}

// Phase B at the leaf level plus the near field: one block per output leaf
// of at most 128 points.
__global__ void __launch_bounds__(THREADS) k_leaf_tc(FarOp op, NearOp nr, const float* __restrict__ T,
                                                     const float* __restrict__ Xt, int64_t N,
                                                     const float* __restrict__ Knear,
                                                     const int64_t* __restrict__ near_off,
                                                     const double* __restrict__ Ynl,
                                                     const int32_t* __restrict__ perm, int nrhs,
                                                     double* __restrict__ Y, int64_t ldy,
                                                     int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[4];
  __shared__ uint32_t tslot;
  __shared__ Item s_items[kMaxItems];
  Engine E;
  engine_setup(E, smem, bar, &tslot, err);
  const int d = op.levels;
  const int64_t k = blockIdx.x;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  const int64_t lk = level_base(d) + k;
  float sum[NR], comp[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) sum[c] = comp[c] = 0.f;
  if (nk > 0) {
    // items: the leaf-level pairs, then the 27 near-field blocks, in batches
    const int64_t q0 = op.il_ptr[lk];
    const int npair = (int)(op.il_ptr[lk + 1] - q0);
    const int total = npair + 27;
    for (int base = 0; base < total; base += kMaxItems) {
      const int nb = min(kMaxItems, total - base);
      __syncthreads();
      for (int i = threadIdx.x; i < nb; i += THREADS) {
        const int g = base + i;
        Item it;
        if (g < npair) {
          const int p = (int)(q0 + g);
          const int r = op.rank[p];
          const int rp = (r + 3) & ~3;
          it.a = static_cast<const float*>(op.ufac[p]);
          it.as = rp;
          it.alen = rp;
          it.b = T + op.tr_off[p] * NR;
          it.bs = r;
          it.blen = r;
        } else {
          const int sl = g - npair;  // neighbour slots 0..25, then the leaf itself
          const int64_t nn = sl < 26 ? (int64_t)nr.nbr_leaf[k * 26 + sl] : k;
          const int64_t off = near_off[k * 27 + sl];
          if (nn >= 0 && off >= 0) {
            const int64_t e0 = op.leaf_off[nn];
            const int ne = (int)(op.leaf_off[nn + 1] - e0);
            const int nep = (ne + 3) & ~3;
            it.a = Knear + off;
            it.as = nep;
            it.alen = nep;
            it.b = Xt + e0;
            it.bs = N;
            it.blen = ne;
          } else {
            it.a = Xt;
            it.b = Xt;
            it.as = it.bs = 0;
            it.alen = it.blen = 0;
          }
        }
        s_items[i] = it;
      }
      __syncthreads();
      long_k(E, s_items, nb, (int)threadIdx.x < nk, sum, comp);
    }
  }
  const int row = threadIdx.x;
  if (row < nk) {
    const int64_t t = t0 + row;
    const int64_t orig = perm[t];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      if (c < nrhs) {
        const double ynl = d >= 2 ? Ynl[(int64_t)c * N + t] : 0.0;
        Y[(int64_t)c * ldy + orig] = ((double)sum[c] - (double)comp[c]) + ynl;
      }
    }
  }
  engine_teardown(E);
}

// X (original order, column-major) -> Xt[c * N + t] in tree order, FP32
__global__ void k_gather_xt(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                            const int32_t* __restrict__ perm, float* __restrict__ Xt) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int c = (int)(o / N);
  const int64_t t = o - (int64_t)c * N;
  Xt[o] = c < nrhs ? (float)X[c * ldx + perm[t]] : 0.f;
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
    Knear[off + e] = v;
  }
}

}  // namespace

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
  k_gather_xt<<<(unsigned)((N * NR + 255) / 256), 256, 0, s>>>(N, nrhs, X, ldx, perm, B.xt);
  ++launches;
  if (prof) prof->mark(s, "gather");
  const int d = far.levels;
  if (d >= 2) {
    const int64_t nslice = int64_t(1) << (3 * (d - 1));
    // spread each slice's row tiles over several blocks when slices are few
    const int split = (int)std::max<int64_t>(1, std::min<int64_t>(16, (8 * 152 + nslice - 1) / nslice));
    k_ta_tc<true><<<dim3((unsigned)nslice, (unsigned)split), THREADS, SMEM_BYTES, s>>>(far, B.xt, N, B.t,
                                                                                    B.p, B.err);
    ++launches;
    if (prof) prof->mark(s, "ta_slice");
    if (B.n_upper > 0) {
      k_tred_tc<<<(unsigned)B.n_upper, 128, 0, s>>>(far, B.upper_pairs, B.p, B.t);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
  }
  k_ta_tc<false><<<dim3((unsigned)far.nleaf, 1), THREADS, SMEM_BYTES, s>>>(far, B.xt, N, B.t, B.p,
                                                                         B.err);
  ++launches;
  if (prof) prof->mark(s, "ta_leaf");
  if (d >= 2) {
    const int64_t nslice = int64_t(1) << (3 * (d - 1));
    const int tiles = (B.max_slice + 127) / 128;
    k_ut_tc<<<dim3((unsigned)nslice, (unsigned)std::max(1, tiles)), THREADS, SMEM_BYTES, s>>>(
        far, B.t, N, B.ynl, B.err);
    ++launches;
    if (prof) prof->mark(s, "ut_tc");
  }
  k_leaf_tc<<<(unsigned)far.nleaf, THREADS, SMEM_BYTES, s>>>(far, near, B.t, B.xt, N, B.knear,
                                                           B.near_off, B.ynl, perm, nrhs, Y, ldy,
                                                           B.err);
  ++launches;
  if (prof) prof->mark(s, "leaf_tc");
  return launches;
}

}  // namespace h3d
