// Host side: factor files (hodlr3d_save / hodlr3d_load).
#include "host.h"

namespace hodlr3d_host {

// ---------------------------------------------------------------------------
// factor files (hodlr3d_save / hodlr3d_load)
// ---------------------------------------------------------------------------
// Version 1, host byte order (little-endian on both supported hosts):
//   "H3DFACT1", FileHeader, points (n x 3 FP64, original order),
//   per pair {rank, pool, offset of U in the pool} (PairRec), the pivots of
//   every pair (rank row then rank column local indices), per pool its FP64
//   element count, the pool contents (per pair U n x r then V m x r,
//   column-major, as the assembly wrote them), a 64-bit checksum of all of it.
// The tree and interaction lists are rebuilt from the points on load and
// must hash to lists_hash: the factors belong to exactly those pairs.
constexpr char kFactMagic[8] = {'H', '3', 'D', 'F', 'A', 'C', 'T', '1'};

struct FileHeader {
  uint32_t version, header_bytes;
  int64_t n;
  int32_t nP1D, tol_pow;
  double L;
  int32_t kernel, levels;
  double diag;
  int64_t npairs;
  int32_t npools, reserved;
  uint64_t lists_hash;
};

struct PairRec {
  int32_t rank, pool;
  int64_t off;
};

// word-wise mixing hash (multiply-xorshift); trailing bytes folded in one word
struct Hasher {
  uint64_t x = 0x243F6A8885A308D3ull;
  void add(const void* p, size_t bytes) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
      uint64_t w;
      std::memcpy(&w, b + i, 8);
      x = (x ^ w) * 0x9E3779B97F4A7C15ull;
      x ^= x >> 29;
    }
    if (i < bytes) {
      uint64_t w = 0;
      std::memcpy(&w, b + i, bytes - i);
      x = (x ^ w ^ (uint64_t)(bytes - i) << 56) * 0x9E3779B97F4A7C15ull;
      x ^= x >> 29;
    }
  }
};

uint64_t lists_hash(const hodlr3d_t h) {
  Hasher hs;
  hs.add(h->h_pair_level.data(), sizeof(int32_t) * h->h_pair_level.size());
  hs.add(h->h_pair_tgt.data(), sizeof(int32_t) * h->h_pair_tgt.size());
  hs.add(h->h_pair_src.data(), sizeof(int32_t) * h->h_pair_src.size());
  hs.add(h->h_leaf_off.data(), sizeof(int32_t) * h->h_leaf_off.size());
  return hs.x;
}

struct File {
  std::FILE* f = nullptr;
  Hasher hs;
  ~File() {
    if (f) std::fclose(f);
  }
  bool write(const void* p, size_t bytes) {
    hs.add(p, bytes);
    return std::fwrite(p, 1, bytes, f) == bytes;
  }
  bool read(void* p, size_t bytes) {
    if (std::fread(p, 1, bytes, f) != bytes) return false;
    hs.add(p, bytes);
    return true;
  }
};

constexpr size_t kFileChunk = size_t(64) << 20;

int save_factors(hodlr3d_t h, const char* path) {
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  const int64_t np = h->npairs;
  // the FP64 pools the pairs use, renumbered in order
  std::vector<int> remap(h->pools.size(), -1), used;
  for (int64_t p = 0; p < np; ++p) {
    const int q = h->h_fac_pool[p];
    if (q >= 0 && remap[q] < 0) {
      remap[q] = 0;
    }
  }
  for (size_t q = 0; q < h->pools.size(); ++q)
    if (remap[q] == 0) {
      remap[q] = (int)used.size();
      used.push_back((int)q);
    }
  File F;
  F.f = std::fopen(path, "wb");
  if (!F.f) return set_error(HODLR3D_ERR_IO, "cannot open %s for writing", path);
  if (std::fwrite(kFactMagic, 1, 8, F.f) != 8) return set_error(HODLR3D_ERR_IO, "write failed: %s", path);
  FileHeader hd{};
  hd.version = 1;
  hd.header_bytes = sizeof(FileHeader);
  hd.n = h->N;
  hd.nP1D = h->nP1D;
  hd.tol_pow = h->tol_pow;
  hd.L = h->L;
  hd.kernel = h->kd.kind;
  hd.levels = h->levels;
  hd.diag = h->kd.diag;
  hd.npairs = np;
  hd.npools = (int32_t)used.size();
  hd.lists_hash = lists_hash(h);
  std::vector<double> xyz(3 * h->N);
  H3D_CUDA(cudaMemcpy(xyz.data(), h->xyz.p, sizeof(double) * xyz.size(), cudaMemcpyDeviceToHost));
  std::vector<PairRec> pr(np);
  for (int64_t p = 0; p < np; ++p)
    pr[p] = {h->h_rank[p], h->h_fac_pool[p] >= 0 ? remap[h->h_fac_pool[p]] : -1, h->h_fac_off[p]};
  bool ok = F.write(&hd, sizeof hd) && F.write(xyz.data(), sizeof(double) * xyz.size()) &&
            F.write(pr.data(), sizeof(PairRec) * pr.size());
  for (int64_t p = 0; ok && p < np; ++p)
    ok = F.write(h->h_piv_rows[p].data(), sizeof(int32_t) * h->h_piv_rows[p].size()) &&
         F.write(h->h_piv_cols[p].data(), sizeof(int32_t) * h->h_piv_cols[p].size());
  std::vector<int64_t> counts;
  for (int q : used) counts.push_back((int64_t)(h->pools[q]->bytes / sizeof(double)));
  ok = ok && F.write(counts.data(), sizeof(int64_t) * counts.size());
  std::vector<unsigned char> buf;
  for (size_t u = 0; ok && u < used.size(); ++u) {
    const DevBuf* b = h->pools[used[u]];
    for (size_t o = 0; ok && o < b->bytes; o += kFileChunk) {
      const size_t len = std::min(kFileChunk, b->bytes - o);
      buf.resize(len);
      H3D_CUDA(cudaMemcpy(buf.data(), static_cast<const unsigned char*>(b->p) + o, len,
                          cudaMemcpyDeviceToHost));
      ok = F.write(buf.data(), len);
    }
  }
  const uint64_t sum = F.hs.x;
  ok = ok && std::fwrite(&sum, 1, 8, F.f) == 8;
  if (!ok || std::fflush(F.f) != 0) return set_error(HODLR3D_ERR_IO, "write failed: %s", path);
  return HODLR3D_OK;
}

int load_factors(const char* path, const hodlr3d_options* opt, hodlr3d_t* out) {
  const double t_start = now_s();
  File F;
  F.f = std::fopen(path, "rb");
  if (!F.f) return set_error(HODLR3D_ERR_IO, "cannot open %s", path);
  char magic[8];
  if (std::fread(magic, 1, 8, F.f) != 8 || std::memcmp(magic, kFactMagic, 8) != 0)
    return set_error(HODLR3D_ERR_IO, "%s is not a hodlr3d factor file (version 1)", path);
  FileHeader hd{};
  // sizes are checked before anything is allocated from them: the point count
  // within what hodlr3d_create takes, at most one pool per pair
  if (!F.read(&hd, sizeof hd) || hd.version != 1 || hd.header_bytes != sizeof(FileHeader) || hd.n < 2 ||
      hd.n > INT32_MAX / 2 || hd.npairs < 0 || hd.npools < 0 || hd.npools > std::max<int64_t>(hd.npairs, 1))
    return set_error(HODLR3D_ERR_IO, "%s: unreadable header", path);
  std::vector<double> xyz(3 * (size_t)hd.n);
  if (!F.read(xyz.data(), sizeof(double) * xyz.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  hodlr3d_options o;
  if (opt) o = *opt;
  else hodlr3d_default_options(&o);
  o.diag_override = hd.diag;
  hodlr3d_t h = nullptr;
  H3D_TRY(hodlr3d_create(xyz.data(), hd.n, hd.nP1D, hd.L, hd.tol_pow, hd.kernel, &o, &h));
  std::unique_ptr<hodlr3d_handle, void (*)(hodlr3d_t)> guard(h, hodlr3d_destroy);
  if (h->levels != hd.levels || h->npairs != hd.npairs || lists_hash(h) != hd.lists_hash)
    return set_error(HODLR3D_ERR_IO, "%s: the tree rebuilt from its points differs from the saved one", path);
  const int64_t np = hd.npairs;
  std::vector<PairRec> pr(np);
  if (!F.read(pr.data(), sizeof(PairRec) * pr.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  h->h_rank.assign(np, 0);
  h->h_piv_rows.assign(np, {});
  h->h_piv_cols.assign(np, {});
  h->h_u64.assign(np, nullptr);
  h->h_v64.assign(np, nullptr);
  h->h_u32.assign(np, nullptr);
  h->h_v32.assign(np, nullptr);
  h->h_fac_pool.assign(np, -1);
  h->h_fac_off.assign(np, 0);
  for (int64_t p = 0; p < np; ++p) {
    const int r = pr[p].rank;
    if (r < 0 || r > h->N || pr[p].pool < -1 || pr[p].pool >= hd.npools || (pr[p].pool < 0 && r > 0))
      return set_error(HODLR3D_ERR_IO, "%s: corrupt pair record %lld", path, (long long)p);
    h->h_rank[p] = r;
    h->h_piv_rows[p].resize(r);
    h->h_piv_cols[p].resize(r);
    if (!F.read(h->h_piv_rows[p].data(), sizeof(int32_t) * r) ||
        !F.read(h->h_piv_cols[p].data(), sizeof(int32_t) * r))
      return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  }
  std::vector<int64_t> counts(hd.npools);
  if (!F.read(counts.data(), sizeof(int64_t) * counts.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  std::vector<unsigned char> buf;
  for (int q = 0; q < hd.npools; ++q) {
    if (counts[q] < 0) return set_error(HODLR3D_ERR_IO, "%s: corrupt pool size", path);
    DevBuf* b = new DevBuf();
    h->pools.push_back(b);
    const size_t bytes = sizeof(double) * (size_t)counts[q];
    H3D_CUDA(b->ensure(bytes));
    for (size_t o = 0; o < bytes; o += kFileChunk) {
      const size_t len = std::min(kFileChunk, bytes - o);
      buf.resize(len);
      if (!F.read(buf.data(), len)) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
      H3D_CUDA(cudaMemcpy(static_cast<unsigned char*>(b->p) + o, buf.data(), len, cudaMemcpyHostToDevice));
    }
  }
  const uint64_t want = F.hs.x;
  uint64_t sum = 0;
  if (std::fread(&sum, 1, 8, F.f) != 8 || sum != want)
    return set_error(HODLR3D_ERR_IO, "%s: checksum mismatch", path);
  for (int64_t p = 0; p < np; ++p) {
    if (pr[p].pool < 0) continue;
    const int j = h->h_pair_level[p];
    int64_t a0, a1, b0, b1;
    box_range(h, j, h->h_pair_tgt[p] - h3d::level_base(j), a0, a1);
    box_range(h, j, h->h_pair_src[p] - h3d::level_base(j), b0, b1);
    const int64_t r = pr[p].rank;
    if (pr[p].off < 0 || pr[p].off + r * ((a1 - a0) + (b1 - b0)) > counts[pr[p].pool])
      return set_error(HODLR3D_ERR_IO, "%s: pair %lld lies outside its pool", path, (long long)p);
    for (int l = 0; l < r; ++l)
      if (h->h_piv_rows[p][l] < 0 || h->h_piv_rows[p][l] >= a1 - a0 || h->h_piv_cols[p][l] < 0 ||
          h->h_piv_cols[p][l] >= b1 - b0)
        return set_error(HODLR3D_ERR_IO, "%s: pivot of pair %lld outside its boxes", path, (long long)p);
    double* base = h->pools[pr[p].pool]->as<double>() + pr[p].off;
    h->h_fac_pool[p] = pr[p].pool;
    h->h_fac_off[p] = pr[p].off;
    h->h_u64[p] = base;
    h->h_v64[p] = base + r * (a1 - a0);
  }
  h->aca_batches = 0;
  h->aca_kernel_seconds = 0.0;
  H3D_TRY(finish_assembly(h, t_start));
  *out = guard.release();
  return HODLR3D_OK;
}

}  // namespace hodlr3d_host
