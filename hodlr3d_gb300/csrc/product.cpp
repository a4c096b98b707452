// Host side: the matvec engines' drivers (CUDA cores, tensor cores, few
// columns), their tables and buffers, and the engine autotuner.
#include "host.h"

namespace hodlr3d_host {

// ---------------------------------------------------------------------------
// matvec
// ---------------------------------------------------------------------------
int ensure_matvec_buffers(hodlr3d_t h, int nrhs) {
  const int nr = h3d::padded_nrhs(nrhs);
  if (nr <= h->mv_nrhs_cap) return HODLR3D_OK;
  H3D_CUDA(h->xsorted.ensure(sizeof(double) * h->N * nr));
  H3D_CUDA(h->tbuf.ensure(sizeof(double) * std::max<int64_t>(h->sum_rank, 1) * nr));
  H3D_CUDA(h->pbuf.ensure(sizeof(double) * std::max<int64_t>(h->part_total, 1) * nr));
  H3D_CUDA(h->ynl.ensure(sizeof(double) * h->N * nr));
  h->mv_nrhs_cap = nr;
  return HODLR3D_OK;
}

// Tensor maps (2D tiled, FP32, 128-byte swizzle, zero fill outside) of the
// tensor-core engine's A operands: per target box the U of its pairs side by
// side (n x R_b) and per source box the V of its pairs (sum of ranks x
// round4(m)), box 32 x 128; per leaf its row matrix (nk x W_k), box 32 x 64.
// Maps of empty operands stay zero and are never used.
int build_tensor_maps(hodlr3d_t h) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    H3D_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&encode, 12000,
                                              cudaEnableDefault, &q));
    if (!encode || q != cudaDriverEntryPointSuccess)
      return set_error(HODLR3D_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  }
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t nm = 2 * nbox + h->nleaf;
  std::vector<CUtensorMap> maps((size_t)std::max<int64_t>(nm, 1));
  std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
  std::atomic<int> bad{0};
  std::mutex bad_mu;
  char bad_msg[160] = {0};
  auto enc = [&](CUtensorMap* m, const float* base, int64_t inner, int64_t rows, uint32_t box_rows,
                 int64_t ld) {
    if (!base || inner <= 0 || rows <= 0) return;
    const cuuint64_t dim[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    const cuuint64_t stride[1] = {(cuuint64_t)ld * sizeof(float)};
    const cuuint32_t box[2] = {32, box_rows}, es[2] = {1, 1};
    const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dim, stride, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS && !bad.exchange(1)) {
      std::lock_guard<std::mutex> g(bad_mu);
      std::snprintf(bad_msg, sizeof(bad_msg), "code %d, %lld x %lld at %p, box 32 x %u, map at %p",
                    (int)r, (long long)rows, (long long)inner, (const void*)base, box_rows, (void*)m);
    }
  };
  const float* krow = h->krow.as<float>();
  const int nthr = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nthr; ++t)
    th.emplace_back([&, t] {
      cudaSetDevice(h->opt.device);  // the encoder wants the device's context current
      for (int64_t b = t; b < nbox; b += nthr) {
        int j = 0;
        while (j < h->levels && h3d::level_base(j + 1) <= b) ++j;
        int64_t b0, b1;
        box_range(h, j, b - h3d::level_base(j), b0, b1);
        if (h->h_rbox[b] > 0)
          enc(&maps[b], h->u32_pool->as<float>() + h->h_ubox_off[b], h->h_rbox[b], b1 - b0, 128,
              h->h_rbox[b]);
        if (h->h_vbox_rows[b] > 0)
          enc(&maps[nbox + b], h->v32_pool->as<float>() + h->h_vbox_off[b],
              ((b1 - b0) + 3) & ~int64_t(3), h->h_vbox_rows[b], 128, ((b1 - b0) + 3) & ~int64_t(3));
      }
      for (int64_t k = t; k < h->nleaf; k += nthr) {
        const int64_t nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
        enc(&maps[2 * nbox + k], krow + h->h_row_base[k], h->h_row_ld[k], nk, 64, h->h_row_ld[k]);
      }
    });
  for (auto& x : th) x.join();
  if (bad) {
    std::lock_guard<std::mutex> g(bad_mu);
    return set_error(HODLR3D_ERR_CUDA, "a tensor map could not be encoded (%s)", bad_msg);
  }
  H3D_CUDA(h->tmaps.ensure(sizeof(CUtensorMap) * maps.size()));
  H3D_CUDA(cudaMemcpy(h->tmaps.p, maps.data(), sizeof(CUtensorMap) * maps.size(),
                      cudaMemcpyHostToDevice));
  h->maps_built = true;
  return HODLR3D_OK;
}

// FP32 near-field blocks of every leaf (both FP32 engines), evaluated once
// per assembly.  The blocks of leaf k (slots 0..25 the neighbours, 26
// itself; absent neighbours skipped) sit side by side in one row-major
// nk x Rn_k matrix at h_near_base[k] (Rn_k = h_near_ld[k], the sum of their
// round4(ne)); slot s's block starts at h_near_off[27 k + s] (-1: absent).
int ensure_near_blocks(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->near_built) return HODLR3D_OK;
  h->h_nbr_leaf.resize(26 * h->nleaf);
  H3D_CUDA(cudaMemcpy(h->h_nbr_leaf.data(), h->nbr_leaf.p, sizeof(int32_t) * 26 * h->nleaf,
                      cudaMemcpyDeviceToHost));
  const std::vector<int32_t>& nbl = h->h_nbr_leaf;
  std::vector<int64_t>& off = h->h_near_off;
  off.assign(27 * h->nleaf, -1);
  h->h_near_base.assign(h->nleaf, 0);
  h->h_near_ld.assign(h->nleaf, 0);
  int64_t tot = 0;
  for (int64_t k = 0; k < h->nleaf; ++k) {
    const int64_t nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
    int64_t col = 0;
    for (int sl = 0; sl < 27; ++sl) {
      const int64_t nn = sl < 26 ? nbl[26 * k + sl] : k;
      if (nn < 0) continue;
      const int64_t ne = h->h_leaf_off[nn + 1] - h->h_leaf_off[nn];
      off[27 * k + sl] = tot + col;
      col += (ne + 3) & ~int64_t(3);
    }
    h->h_near_base[k] = tot;
    h->h_near_ld[k] = (int32_t)col;
    tot += nk * col;
  }
  H3D_CUDA(h->knear.ensure(sizeof(float) * std::max<int64_t>(tot, 4)));
  H3D_CUDA(h->near_off.ensure(sizeof(int64_t) * off.size()));
  H3D_CUDA(cudaMemcpy(h->near_off.p, off.data(), sizeof(int64_t) * off.size(),
                      cudaMemcpyHostToDevice));
  H3D_CUDA(h->near_base.ensure(sizeof(int64_t) * h->nleaf));
  H3D_CUDA(cudaMemcpy(h->near_base.p, h->h_near_base.data(), sizeof(int64_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  H3D_CUDA(h->near_ld.ensure(sizeof(int32_t) * h->nleaf));
  H3D_CUDA(cudaMemcpy(h->near_ld.p, h->h_near_ld.data(), sizeof(int32_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  h->launches += h3d::launch_near_blocks(s, h->nleaf, h->leaf_off.as<int32_t>(), nr,
                                         h->near_off.as<int64_t>(), h->near_ld.as<int32_t>(),
                                         h->knear.as<float>());
  H3D_CUDA(cudaGetLastError());
  h->near_floats = tot;
  h->near_built = true;
  return HODLR3D_OK;
}

// Leaf rows of the tensor-core engine: for every leaf (at most 64 points) its
// blocks -- near field (neighbour slots 0..25 with a leaf, then itself), then
// its leaf-level interaction list in pair order -- each nk x round4(m), side
// by side in one row-major nk x W_k FP32 matrix, evaluated once per handle
// (they depend on the points only).
int ensure_leaf_rows(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->rows_built) return HODLR3D_OK;
  if ((int64_t)h->h_nbr_leaf.size() != 26 * h->nleaf) {
    h->h_nbr_leaf.resize(26 * h->nleaf);
    H3D_CUDA(cudaMemcpy(h->h_nbr_leaf.data(), h->nbr_leaf.p, sizeof(int32_t) * 26 * h->nleaf,
                        cudaMemcpyDeviceToHost));
  }
  const int d = h->levels;
  const int64_t lb = h3d::level_base(d);
  std::vector<h3d::LeafBlock> blocks;
  std::vector<int32_t> ptr(h->nleaf + 1, 0);
  h->h_row_base.assign(h->nleaf, 0);
  h->h_row_ld.assign(h->nleaf, 0);
  int64_t tot = 0;
  int maxb = 0;
  for (int64_t k = 0; k < h->nleaf; ++k) {
    const int64_t nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
    int64_t col = 0;
    auto add = [&](int64_t src) {
      const int64_t m = h->h_leaf_off[src + 1] - h->h_leaf_off[src];
      if (m <= 0) return;
      blocks.push_back({(int32_t)col, h->h_leaf_off[src], (int32_t)m, (int32_t)src});
      col += (m + 3) & ~int64_t(3);
    };
    for (int sl = 0; sl < 27; ++sl) {
      const int64_t nn = sl < 26 ? h->h_nbr_leaf[26 * k + sl] : k;
      if (nn >= 0) add(nn);
    }
    if (d >= 1)
      for (int64_t p = h->h_il_ptr[lb + k]; p < h->h_il_ptr[lb + k + 1]; ++p) add(h->h_pair_src[p] - lb);
    ptr[k + 1] = (int32_t)blocks.size();
    maxb = std::max(maxb, ptr[k + 1] - ptr[k]);
    if (maxb > h3d::tc_max_row_blocks())
      return set_error(HODLR3D_ERR_UNSUPPORTED, "a leaf row has %d blocks; the tensor-core engine takes %d",
                       maxb, h3d::tc_max_row_blocks());
    if (col >= INT32_MAX) return set_error(HODLR3D_ERR_UNSUPPORTED, "leaf row wider than 2^31 - 1");
    h->h_row_base[k] = tot;
    h->h_row_ld[k] = (int32_t)col;
    tot += nk * col;
  }
  H3D_CUDA(h->krow.ensure(sizeof(float) * std::max<int64_t>(tot, 4)));
  H3D_CUDA(h->leaf_blocks.ensure(sizeof(h3d::LeafBlock) * std::max<size_t>(blocks.size(), 1)));
  H3D_CUDA(h->block_ptr.ensure(sizeof(int32_t) * ptr.size()));
  H3D_CUDA(h->row_base.ensure(sizeof(int64_t) * std::max<int64_t>(h->nleaf, 1)));
  H3D_CUDA(h->row_ld.ensure(sizeof(int32_t) * std::max<int64_t>(h->nleaf, 1)));
  if (!blocks.empty())
    H3D_CUDA(cudaMemcpy(h->leaf_blocks.p, blocks.data(), sizeof(h3d::LeafBlock) * blocks.size(),
                        cudaMemcpyHostToDevice));
  H3D_CUDA(cudaMemcpy(h->block_ptr.p, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice));
  H3D_CUDA(cudaMemcpy(h->row_base.p, h->h_row_base.data(), sizeof(int64_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  H3D_CUDA(cudaMemcpy(h->row_ld.p, h->h_row_ld.data(), sizeof(int32_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  h->launches += h3d::launch_row_blocks(s, h->nleaf, maxb, h->leaf_off.as<int32_t>(), nr,
                                        h->leaf_blocks.as<h3d::LeafBlock>(), h->block_ptr.as<int32_t>(),
                                        h->row_base.as<int64_t>(), h->row_ld.as<int32_t>(),
                                        h->krow.as<float>());
  H3D_CUDA(cudaGetLastError());
  h->max_blocks = maxb;
  h->row_floats = tot;
  h->rows_built = true;
  h->maps_built = false;
  return HODLR3D_OK;
}

// Work lists and index tables of the few-column engine (matvec_gemv.cu) over
// the grouped FP32 layouts; leaves it off (gemv_ok false) when the tree does
// not fit its shared memory or 32-bit row numbers.
int ensure_gemv(hodlr3d_t h, cudaStream_t s) {
  if (h->gemv_built) return HODLR3D_OK;
  h->gemv_built = true;
  h->gemv_ok = false;
  const int ml4 = (h->max_leaf + 3) & ~3;
  if (h3d::gemv_smem_bytes(ml4, 4, true) > 200 * 1024) return HODLR3D_OK;
  const int64_t np = h->npairs;
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t trows = h->h_tbox_off[nbox] / 32;
  std::vector<int64_t> vrow0(nbox + 1, 0), tbase(nbox, 0), vpofs(nbox, -1), upofs(nbox, -1);
  for (int64_t b = 0; b < nbox; ++b) {
    tbase[b] = h->h_tbox_off[b] / 32;
    vrow0[b + 1] = vrow0[b] + h->h_vbox_rows[b];
  }
  const int64_t vrows = vrow0[nbox];
  if (trows >= INT32_MAX || vrows >= INT32_MAX) return HODLR3D_OK;
  std::vector<int32_t> rev(std::max<int64_t>(np, 1)), tgt(std::max<int64_t>(np, 1));
  if (np) H3D_CUDA(cudaMemcpy(rev.data(), h->rev.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
  for (int64_t b = 0; b < nbox; ++b)
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p) tgt[p] = (int32_t)b;
  std::vector<int32_t> vrow_t(std::max<int64_t>(vrows, 1)), trow_v(std::max<int64_t>(trows, 1), -1);
  std::vector<int32_t> vt_upper, ut_upper;
  std::vector<int32_t> vt_items, ut_items;  // int4 / int2 records
  int64_t pv = 0, pu = 0;
  for (int64_t b = 0; b < nbox; ++b) {
    int j = 0;
    while (j < h->levels && h3d::level_base(j + 1) <= b) ++j;
    int64_t a0, a1;
    box_range(h, j, b - h3d::level_base(j), a0, a1);
    const int64_t m = a1 - a0, m4 = (m + 3) & ~int64_t(3);
    // V stack of b as a source box: rows map to T rows of the pairs' targets
    int64_t v = vrow0[b];
    for (int64_t q = h->h_il_ptr[b]; q < h->h_il_ptr[b + 1]; ++q) {
      const int p = rev[q];
      const int64_t base = tbase[tgt[p]] + h->h_coff[p];
      for (int l = 0; l < h->h_rank[p]; ++l) {
        trow_v[base + l] = (int32_t)v;
        vrow_t[v++] = (int32_t)(base + l);
      }
    }
    const int rows = h->h_vbox_rows[b];
    if (rows > 0 && m > 0) {
      const int nch = (int)((m4 + h3d::kGemvCols - 1) / h3d::kGemvCols);
      if (nch > 1) {
        vpofs[b] = pv;
        pv += (int64_t)rows * nch;
        vt_upper.push_back((int32_t)b);
      }
      for (int ci = 0; ci < nch; ++ci)
        for (int r0 = 0; r0 < rows; r0 += h3d::kGemvRowChunk) {
          const int rec[4] = {(int32_t)b, ci, r0, std::min(h3d::kGemvRowChunk, rows - r0)};
          vt_items.insert(vt_items.end(), rec, rec + 4);
        }
    }
    // U of b as a target box
    const int R = h->h_rbox[b];
    if (R > 0 && m > 0) {
      const int nch = (int)((m + h3d::kGemvRowsT - 1) / h3d::kGemvRowsT);
      if (nch > 1) {
        upofs[b] = pu;
        pu += (int64_t)R * nch;
        ut_upper.push_back((int32_t)b);
      }
      for (int ci = 0; ci < nch; ++ci) {
        ut_items.push_back((int32_t)b);
        ut_items.push_back(ci);
      }
    }
  }
  auto put = [](DevBuf& d, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = d.ensure(std::max<size_t>(bytes, 16));
    if (e != cudaSuccess || bytes == 0) return e;
    return cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice);
  };
  H3D_CUDA(put(h->gv_ubox_off, h->h_ubox_off.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vbox_off, h->h_vbox_off.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vbox_rows, h->h_vbox_rows.data(), sizeof(int32_t) * nbox));
  H3D_CUDA(put(h->gv_vrow0, vrow0.data(), sizeof(int64_t) * (nbox + 1)));
  H3D_CUDA(put(h->gv_vrow_t, vrow_t.data(), sizeof(int32_t) * vrows));
  H3D_CUDA(put(h->gv_trow_v, trow_v.data(), sizeof(int32_t) * trows));
  H3D_CUDA(put(h->gv_tbase, tbase.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vpofs, vpofs.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_upofs, upofs.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vt_items, vt_items.data(), sizeof(int32_t) * vt_items.size()));
  H3D_CUDA(put(h->gv_vt_upper, vt_upper.data(), sizeof(int32_t) * vt_upper.size()));
  H3D_CUDA(put(h->gv_ut_items, ut_items.data(), sizeof(int32_t) * ut_items.size()));
  H3D_CUDA(put(h->gv_ut_upper, ut_upper.data(), sizeof(int32_t) * ut_upper.size()));
  h->gv_trows = trows;
  h->gv_vrows = vrows;
  h->gv_pv = pv;
  h->gv_pu = pu;
  h->gv_n_vt_items = (int64_t)vt_items.size() / 4;
  h->gv_n_vt_upper = (int64_t)vt_upper.size();
  h->gv_n_ut_items = (int64_t)ut_items.size() / 2;
  h->gv_n_ut_upper = (int64_t)ut_upper.size();
  // 8 columns (mixed); the fp64x form's 4 columns of FP32 pairs fit too
  H3D_CUDA(h->gv_x.ensure(sizeof(float) * 8 * h->N));
  H3D_CUDA(h->gv_t.ensure(sizeof(float) * 8 * std::max<int64_t>(trows, 1)));
  H3D_CUDA(cudaMemsetAsync(h->gv_t.p, 0, sizeof(float) * 8 * std::max<int64_t>(trows, 1), s));
  H3D_CUDA(h->gv_tt.ensure(sizeof(float) * 8 * std::max<int64_t>(vrows, 1)));
  H3D_CUDA(h->gv_p.ensure(sizeof(float) * 8 * std::max<int64_t>(pv, 1)));
  H3D_CUDA(h->gv_pt.ensure(sizeof(float) * 8 * std::max<int64_t>(pu, 1)));
  h->gemv8_ok = h3d::gemv_smem_bytes(ml4, 8, false) <= 200 * 1024;
  h->gemv_ok = true;
  return HODLR3D_OK;
}

// The FP64-accurate form's lo parts (U, V, near field) and its work buffers,
// built on first use after each assembly.
int ensure_lo(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->lo_built) return HODLR3D_OK;
  const int64_t np = h->npairs;
  const float* ubase = h->u32_pool->as<float>();
  const float* vbase = h->v32_pool->as<float>();
  H3D_CUDA(h->u32lo_pool.ensure(h->u32_pool->bytes));
  H3D_CUDA(h->v32lo_pool.ensure(h->v32_pool->bytes));
  if (np) {
    std::vector<float*> ulo(np), vlo(np);
    for (int64_t p = 0; p < np; ++p) {
      ulo[p] = h->u32lo_pool.as<float>() + (h->h_u32[p] - ubase);
      vlo[p] = h->v32lo_pool.as<float>() + (h->h_v32[p] - vbase);
    }
    DevBuf d64, dlo, dsz, dr, dus;
    H3D_CUDA(d64.ensure(sizeof(void*) * np));
    H3D_CUDA(dlo.ensure(sizeof(void*) * np));
    H3D_CUDA(dsz.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dr.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dus.ensure(sizeof(int32_t) * np));
    H3D_CUDA(cudaMemcpy(dr.p, h->h_rank.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dus.p, h->h_ustride.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    // V
    H3D_CUDA(cudaMemcpy(d64.p, h->h_v64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dlo.p, vlo.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dsz.p, h->h_pair_m.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(h3d::launch_v32(s, np, d64.as<const double* const>(), dlo.as<float* const>(),
                             dsz.as<int32_t>(), dr.as<int32_t>(), 1));
    H3D_CUDA(cudaStreamSynchronize(s));
    // U
    H3D_CUDA(cudaMemcpy(d64.p, h->h_u64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dlo.p, ulo.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dsz.p, h->h_pair_n.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(h3d::launch_u32(s, np, d64.as<const double* const>(), dlo.as<float* const>(),
                             dsz.as<int32_t>(), dus.as<int32_t>(), dr.as<int32_t>(), 1));
    H3D_CUDA(cudaStreamSynchronize(s));
    h->launches += 2;
  }
  H3D_CUDA(h->knearlo.ensure(sizeof(float) * std::max<int64_t>(h->near_floats, 4)));
  h->launches += h3d::launch_near_lo(s, h->nleaf, h->leaf_off.as<int32_t>(), nr,
                                     h->near_off.as<int64_t>(), h->near_ld.as<int32_t>(),
                                     h->knear.as<float>(), h->knearlo.as<float>());
  H3D_CUDA(cudaGetLastError());
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t trows = std::max<int64_t>(h->h_tbox_off[nbox] / 32, 1);
  const size_t gp = h->gv_p.bytes / sizeof(float), gpt = h->gv_pt.bytes / sizeof(float);
  H3D_CUDA(h->gv_xl.ensure(sizeof(float) * 4 * h->N));
  H3D_CUDA(h->gv_tl.ensure(sizeof(float) * 4 * trows));
  H3D_CUDA(cudaMemsetAsync(h->gv_tl.p, 0, sizeof(float) * 4 * trows, s));
  H3D_CUDA(h->gv_ttl.ensure(h->gv_tt.bytes));
  H3D_CUDA(h->gv_pd.ensure(sizeof(double) * gp));
  H3D_CUDA(h->gv_ptd.ensure(sizeof(double) * gpt));
  h->lo_built = true;
  return HODLR3D_OK;
}

// The FP64 streaming engine's grouped FP64 factors, FP64 near-field blocks
// and work buffers, built on first use after each assembly (the few-column
// tables exist).  When they do not fit in device memory the engine is left
// out for this assembly and the CUDA-core FP64 kernels serve.
int ensure_f64(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->f64_built || h->f64_unavailable) return HODLR3D_OK;
  const int64_t np = h->npairs;
  auto release = [&] {
    cudaGetLastError();
    for (DevBuf* b : {&h->u64g_pool, &h->v64g_pool, &h->knear64, &h->f64_x, &h->f64_t, &h->f64_tt,
                      &h->f64_p, &h->f64_pt})
      b->release();
    h->f64_unavailable = true;
  };
  auto get = [&](DevBuf& b, size_t bytes) {
    const cudaError_t e = b.ensure(std::max<size_t>(bytes, 16));
    return e;
  };
  const size_t ub = h->u32_pool->bytes / sizeof(float) * sizeof(double);
  const size_t vb = h->v32_pool->bytes / sizeof(float) * sizeof(double);
  for (auto& req : std::vector<std::pair<DevBuf*, size_t>>{
           {&h->u64g_pool, ub},
           {&h->v64g_pool, vb},
           {&h->knear64, sizeof(double) * (size_t)std::max<int64_t>(h->near_floats, 4)},
           {&h->f64_x, sizeof(double) * (size_t)h->N},
           {&h->f64_t, sizeof(double) * (size_t)std::max<int64_t>(h->gv_trows, 1)},
           {&h->f64_tt, sizeof(double) * (size_t)std::max<int64_t>(h->gv_vrows, 1)},
           {&h->f64_p, sizeof(double) * (size_t)std::max<int64_t>(h->gv_pv, 1)},
           {&h->f64_pt, sizeof(double) * (size_t)std::max<int64_t>(h->gv_pu, 1)}}) {
    const cudaError_t e = get(*req.first, req.second);
    if (e == cudaErrorMemoryAllocation) {
      release();
      return HODLR3D_OK;
    }
    H3D_CUDA(e);
  }
  H3D_CUDA(cudaMemsetAsync(h->f64_t.p, 0, h->f64_t.bytes, s));
  if (np) {
    const float* ubase = h->u32_pool->as<float>();
    const float* vbase = h->v32_pool->as<float>();
    std::vector<double*> ug(np), vg(np);
    for (int64_t p = 0; p < np; ++p) {
      ug[p] = h->u64g_pool.as<double>() + (h->h_u32[p] - ubase);
      vg[p] = h->v64g_pool.as<double>() + (h->h_v32[p] - vbase);
    }
    DevBuf du, dv, dug, dvg, dn, dm, dus, dr;
    H3D_CUDA(du.ensure(sizeof(void*) * np));
    H3D_CUDA(dv.ensure(sizeof(void*) * np));
    H3D_CUDA(dug.ensure(sizeof(void*) * np));
    H3D_CUDA(dvg.ensure(sizeof(void*) * np));
    H3D_CUDA(dn.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dm.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dus.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dr.ensure(sizeof(int32_t) * np));
    H3D_CUDA(cudaMemcpy(du.p, h->h_u64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dv.p, h->h_v64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dug.p, ug.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dvg.p, vg.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dn.p, h->h_pair_n.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dm.p, h->h_pair_m.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dus.p, h->h_ustride.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dr.p, h->h_rank.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    h->launches += h3d::launch_group_f64(s, np, du.as<const double* const>(), dug.as<double* const>(),
                                         dn.as<int32_t>(), dus.as<int32_t>(), dv.as<const double* const>(),
                                         dvg.as<double* const>(), dm.as<int32_t>(), dr.as<int32_t>());
    H3D_CUDA(cudaGetLastError());
    H3D_CUDA(cudaStreamSynchronize(s));
  }
  h->launches += h3d::launch_near64(s, h->nleaf, h->leaf_off.as<int32_t>(), nr, h->near_off.as<int64_t>(),
                                    h->near_ld.as<int32_t>(), h->knear64.as<double>());
  H3D_CUDA(cudaGetLastError());
  h->f64_built = true;
  return HODLR3D_OK;
}

h3d::GemvOp gemv_op(hodlr3d_t h, bool fp64x);

// The FP64 streaming engine (matvec_f64.cu), one column per pass.
int run_f64(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, cudaStream_t s, bool trans) {
  const h3d::GemvOp g = gemv_op(h, false);
  h3d::F64Buffers B{};
  B.u64 = h->u64g_pool.as<double>();
  B.v64 = h->v64g_pool.as<double>();
  B.knear64 = h->knear64.as<double>();
  B.xg = h->f64_x.as<double>();
  B.t = h->f64_t.as<double>();
  B.tt = h->f64_tt.as<double>();
  B.p = h->f64_p.as<double>();
  B.pt = h->f64_pt.as<double>();
  B.vt_items = h->gv_vt_items.as<int4>();
  B.n_vt_items = h->gv_n_vt_items;
  B.vt_upper = h->gv_vt_upper.as<int32_t>();
  B.n_vt_upper = h->gv_n_vt_upper;
  B.ut_items = h->gv_ut_items.as<int2>();
  B.n_ut_items = h->gv_n_ut_items;
  B.ut_upper = h->gv_ut_upper.as<int32_t>();
  B.n_ut_upper = h->gv_n_ut_upper;
  for (int c = 0; c < nrhs; ++c)
    h->launches += h3d::launch_matvec_f64(s, g, B, x + c * ld, y + c * ld, trans,
                                          h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// The few-column engine (matvec_gemv.cu) over this handle's tables, in passes
// of 4 (or 8) columns; its tables and, for fp64x, the lo parts exist.
h3d::GemvOp gemv_op(hodlr3d_t h, bool fp64x) {
  h3d::GemvOp g{};
  g.levels = h->levels;
  g.max_leaf4 = (h->max_leaf + 3) & ~3;
  g.nleaf = h->nleaf;
  g.N = h->N;
  g.leaf_off = h->leaf_off.as<int32_t>();
  g.perm = h->perm.as<int32_t>();
  g.nbr_leaf = h->nbr_leaf.as<int32_t>();
  g.u32 = h->u32_pool->as<float>();
  g.v32 = h->v32_pool->as<float>();
  g.ubox_off = h->gv_ubox_off.as<int64_t>();
  g.rbox = h->tc_rbox.as<int32_t>();
  g.vbox_off = h->gv_vbox_off.as<int64_t>();
  g.vbox_rows = h->gv_vbox_rows.as<int32_t>();
  g.vrow0 = h->gv_vrow0.as<int64_t>();
  g.vrow_t = h->gv_vrow_t.as<int32_t>();
  g.trow_v = h->gv_trow_v.as<int32_t>();
  g.tbase = h->gv_tbase.as<int64_t>();
  g.vpofs = h->gv_vpofs.as<int64_t>();
  g.upofs = h->gv_upofs.as<int64_t>();
  g.knear = h->knear.as<float>();
  g.u32lo = fp64x ? h->u32lo_pool.as<float>() : nullptr;
  g.v32lo = fp64x ? h->v32lo_pool.as<float>() : nullptr;
  g.knearlo = fp64x ? h->knearlo.as<float>() : nullptr;
  g.near_base = h->near_base.as<int64_t>();
  g.near_ld = h->near_ld.as<int32_t>();
  g.near_off = h->near_off.as<int64_t>();
  return g;
}

int run_gemv(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, cudaStream_t s,
             bool trans, bool fp64x) {
  const h3d::GemvOp g = gemv_op(h, fp64x);
  h3d::GemvBuffers gb{};
  gb.xg = h->gv_x.as<float>();
  gb.t = h->gv_t.as<float>();
  gb.tt = h->gv_tt.as<float>();
  gb.p = h->gv_p.as<float>();
  gb.pt = h->gv_pt.as<float>();
  gb.xl = h->gv_xl.as<float>();
  gb.tl = h->gv_tl.as<float>();
  gb.ttl = h->gv_ttl.as<float>();
  gb.pd = h->gv_pd.as<double>();
  gb.ptd = h->gv_ptd.as<double>();
  gb.vt_items = h->gv_vt_items.as<int4>();
  gb.n_vt_items = h->gv_n_vt_items;
  gb.vt_upper = h->gv_vt_upper.as<int32_t>();
  gb.n_vt_upper = h->gv_n_vt_upper;
  gb.ut_items = h->gv_ut_items.as<int2>();
  gb.n_ut_items = h->gv_n_ut_items;
  gb.ut_upper = h->gv_ut_upper.as<int32_t>();
  gb.n_ut_upper = h->gv_n_ut_upper;
  // passes of 8 columns for the mixed transpose (when the leaves'
  // near-field inputs fit the shared memory: 8 columns 11.6 ms against two
  // passes of 4, 14.1 ms, at 64^3), else of 4 (the forward kernels read the
  // vector with a lane stride of 4 NR floats, which 8 columns turn into
  // serialised shared-memory and L1 accesses: 16.8 ms against 11.4)
  const int width = (!fp64x && trans && nrhs > 4 && h->gemv8_ok) ? 8 : 4;
  for (int c0 = 0; c0 < nrhs; c0 += width)
    h->launches += h3d::launch_matvec_gemv(s, g, gb, x + c0 * ld, ld, y + c0 * ld, ld,
                                           std::min(width, nrhs - c0), trans, fp64x,
                                           h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// The tensor-core engine (matvec_tc.cu) in batches of 32 columns; builds its
// leaf rows and tensor maps on first use.
int run_tc(hodlr3d_t h, const h3d::FarOp& far, const h3d::NearOp& nr, const double* x, double* y,
           int nrhs, int64_t ld, cudaStream_t s) {
  H3D_TRY(ensure_matvec_buffers(h, 32));  // slice partials and level sums of 32 columns
  if (!h->dev_err.p) {
    H3D_CUDA(h->dev_err.ensure(sizeof(int)));
    H3D_CUDA(cudaMemsetAsync(h->dev_err.p, 0, sizeof(int), s));
  }
  H3D_TRY(ensure_leaf_rows(h, nr, s));
  if (!h->maps_built) H3D_TRY(build_tensor_maps(h));
  // [X | T | X_lo | T_lo], the B operands in the split-exact form and their
  // low parts (v - v with the 13 low mantissa bits cleared)
  const int64_t xt_floats = 32 * (h->N + std::max<int64_t>(h->sum_rank4, 1));
  H3D_CUDA(h->tct.ensure(sizeof(float) * 2 * xt_floats));
  h3d::TcBuffers T{};
  T.xt = h->tct.as<float>();
  T.t = T.xt + 32 * h->N;
  T.lo_off = xt_floats;
  T.ta_split = h->tc_split;
  T.p = reinterpret_cast<float*>(h->pbuf.p);
  T.ynl = h->ynl.as<double>();
  T.err = h->dev_err.as<int>();
  T.upper_pairs = h->upper.as<int32_t>();
  T.n_upper = h->n_upper;
  T.max_slice = h->max_slice;
  T.blocks = h->leaf_blocks.as<h3d::LeafBlock>();
  T.block_ptr = h->block_ptr.as<int32_t>();
  const CUtensorMap* tm = h->tmaps.as<CUtensorMap>();
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  T.umaps = tm;
  T.vmaps = tm + nbox;
  T.rmaps = tm + 2 * nbox;
  for (int c0 = 0; c0 < nrhs; c0 += 32)
    h->launches += h3d::launch_matvec_tc(s, h->N, h->perm.as<int32_t>(), far, nr, T, x + c0 * ld,
                                         ld, y + c0 * ld, ld, std::min(32, nrhs - c0),
                                         h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// largest column counts the few-column engine takes in the automatic choice
// (measured at 64^3: 5.7 ms for 4 columns and 11.3 ms for 8 against 6.9 ms
// for the tensor cores' 32; transposed, 7.0 ms for 4 and 46 ms for 32
// columns against 28 and 53 ms for the CUDA-core transpose)
constexpr int kGemvForwardMax = 4;
constexpr int kGemvTransposeMax = 32;
// on trees the tensor-core engine does not take, passes of 4 columns beat the
// CUDA-core kernels' single pass up to 32 columns (64^3: ~6 ms per pass
// against 54 ms for 32 columns)
constexpr int kGemvForwardNoTcMax = 32;

// The operator as the matvec kernels see it: pair tables and factors (FP32
// copies when f32, else the FP64 factors), and the near field.
h3d::FarOp far_op(hodlr3d_t h, bool f32) {
  h3d::FarOp far{};
  far.levels = h->levels;
  far.nleaf = h->nleaf;
  far.leaf_off = h->leaf_off.as<int32_t>();
  far.il_ptr = h->il_ptr.as<int64_t>();
  far.rev = h->rev.as<int32_t>();
  far.rank = h->rank.as<int32_t>();
  far.pair_level = h->pair_level.as<int32_t>();
  far.pair_tgt = h->pair_tgt.as<int32_t>();
  far.pair_src = h->pair_src.as<int32_t>();
  far.tr_off = h->tr_off.as<int64_t>();
  far.ustride = h->ustride.as<int32_t>();
  far.tc_toff = h->tc_toff.as<int64_t>();
  far.tc_tld = h->tc_tld.as<int32_t>();
  far.tc_tbox = h->tc_tbox.as<int64_t>();
  far.tc_rbox = h->tc_rbox.as<int32_t>();
  far.part_off = h->part_off.as<int64_t>();
  far.ufac = f32 ? h->u32.as<const void*>() : h->u64.as<const void*>();
  far.vfac = f32 ? h->v32.as<const void*>() : h->v64.as<const void*>();
  return far;
}

h3d::NearOp near_op(hodlr3d_t h) {
  h3d::NearOp nr{};
  nr.nbr_leaf = h->nbr_leaf.as<int32_t>();
  nr.xs = h->xs.as<double>();
  nr.ys = h->ys.as<double>();
  nr.zs = h->zs.as<double>();
  nr.xl = h->xl.as<float>();
  nr.yl = h->yl.as<float>();
  nr.zl = h->zl.as<float>();
  nr.centre = h->centre.as<double>();
  nr.kd = h->kd;
  return nr;
}

int matvec_device(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, int precision,
                  cudaStream_t s, bool trans) {
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!x || !y) return set_error(HODLR3D_ERR_INVALID_ARG, "null vector");
  if (nrhs < 1 || nrhs > 64) return set_error(HODLR3D_ERR_INVALID_ARG, "nrhs must be in 1..64");
  if (ld < h->N) return set_error(HODLR3D_ERR_INVALID_ARG, "ld < n");
  if (precision != HODLR3D_FP64 && precision != HODLR3D_MIXED && precision != HODLR3D_FP64X)
    return set_error(HODLR3D_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (precision == HODLR3D_MIXED && !h->opt.keep_fp32)
    return set_error(HODLR3D_ERR_INVALID_ARG, "mixed precision needs keep_fp32");
  // the FP64-accurate form builds on the FP32 copies; without them, or on a
  // tree the few-column kernels do not take, it is the FP64 form
  if (precision == HODLR3D_FP64X && !h->opt.keep_fp32) precision = HODLR3D_FP64;
  H3D_TRY(ensure_matvec_buffers(h, nrhs));
  const bool f32 = precision == HODLR3D_MIXED;
  h3d::FarOp far = far_op(h, f32);
  const h3d::NearOp nr = near_op(h);
  h3d::MatvecBuffers B{};
  B.xsorted = h->xsorted.p;
  B.tbuf = h->tbuf.p;
  B.pbuf = h->pbuf.as<double>();
  B.ynl = h->ynl.as<double>();
  B.items = h->items.as<int32_t>();
  B.n_items = h->n_items;
  B.upper_pairs = h->upper.as<int32_t>();
  B.n_upper = h->n_upper;
  B.max_slice = h->max_slice;
  // Mixed form: the few-column engine streams the FP32 factors once per 4
  // right-hand sides; the tensor-core engine once per 32 at a higher cost per
  // factor entry, so it takes the forward product from kGemvForwardMax + 1
  // columns on.  The transpose has no tensor-core form: past
  // kGemvTransposeMax columns the CUDA-core kernels (all columns in one pass)
  // are faster.
  const bool mixed = precision == HODLR3D_MIXED;
  const bool fp64x = precision == HODLR3D_FP64X;
  // the engine of this call: forced, tuned (automatic choice after
  // hodlr3d_autotune, mixed form) or 0 for the rules below
  const int engine = h->engine == 0 && mixed ? h->tuned[trans ? 1 : 0][nrhs] : h->engine;
  // trees the tensor-core engine takes (leaves of at most 64 points, 16-byte
  // aligned leaf rows, bounded tables)
  const bool tc_tree = h->max_leaf <= 64 && h->leaves_aligned && h->tc_entries <= h3d::tc_max_entries();
  const int gemv_max = trans ? kGemvTransposeMax : (tc_tree ? kGemvForwardMax : kGemvForwardNoTcMax);
  bool use_gemv = false;
  // fp64x: the few-column kernels (automatic or forced); forcing the CUDA-core
  // kernels gives the FP64 form; the tensor cores have no FP64-accurate form
  if (fp64x && engine == 2)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the tensor-core engine has no FP64-accurate form (use HODLR3D_MIXED or "
                     "another engine)");
  if ((fp64x && engine != 1) ||
      (mixed && (engine == 3 || (engine == 0 && nrhs <= gemv_max)))) {
    H3D_TRY(ensure_near_blocks(h, nr, s));
    H3D_TRY(ensure_gemv(h, s));
    use_gemv = h->gemv_ok;
    if (use_gemv && fp64x && !h->lo_unavailable) {
      const int st = ensure_lo(h, nr, s);
      if (st == HODLR3D_ERR_OUT_OF_MEMORY) {
        // the lo parts (as large as the FP32 copies) do not fit: the FP64 form
        // serves instead, now and for the rest of this assembly
        cudaGetLastError();
        h->u32lo_pool.release();
        h->v32lo_pool.release();
        h->knearlo.release();
        h->lo_unavailable = true;
      } else if (st != HODLR3D_OK) {
        return st;
      }
    }
    if (fp64x && h->lo_unavailable) use_gemv = false;
  }
  if (fp64x && !use_gemv) {
    precision = HODLR3D_FP64;
    far = far_op(h, false);
  }
  // the FP64 form: streamed from FP64 copies grouped like the FP32 ones
  // (automatic or forced few-column engine); else the CUDA-core kernels
  // (its grouped layout is the FP32 copies' one: with keep_fp32 = 0 there is none)
  if (precision == HODLR3D_FP64 && !use_gemv && h->opt.keep_fp32 && (engine == 0 || engine == 3)) {
    H3D_TRY(ensure_near_blocks(h, nr, s));
    H3D_TRY(ensure_gemv(h, s));
    if (h->gemv_ok) {
      H3D_TRY(ensure_f64(h, nr, s));
      if (h->f64_built) return run_f64(h, x, y, nrhs, ld, s, trans);
    }
    if (engine == 3)
      return set_error(HODLR3D_ERR_UNSUPPORTED,
                       "the few-column engine's FP64 form needs leaves whose near-field inputs fit "
                       "its shared memory, fewer than 2^31 rows of T and device memory for the FP64 "
                       "factors grouped by box");
  }
  if (engine == 3 && !use_gemv && !fp64x)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the few-column engine needs the mixed or FP64 form, leaves whose near-field "
                     "inputs fit its shared memory and fewer than 2^31 rows of T");
  if (use_gemv) return run_gemv(h, x, y, nrhs, ld, s, trans, fp64x);
  const bool tc_ok = mixed && !trans && tc_tree;
  if (engine == 2 && !tc_ok)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the tensor-core engine needs A x (not the transpose) in the mixed form, "
                     "leaves of at most 64 points, each a multiple of 4, and at most %d pairs per "
                     "block (this tree: %d)", h3d::tc_max_entries(), h->tc_entries);
  if (tc_ok && engine != 1) return run_tc(h, far, nr, x, y, nrhs, ld, s);
  // the CUDA-core engine (matvec.cu)
  h->launches += h3d::launch_matvec(s, h->N, h->perm.as<int32_t>(), far, nr, B, x, ld, y, ld, nrhs,
                                    precision, trans ? 1 : 0, h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// ---------------------------------------------------------------------------
// autotuning of the automatic engine choice
// ---------------------------------------------------------------------------
// Column counts timed; a count between two of them takes the choice of the
// next one up (the engines' costs step at powers of two: the tensor cores pad
// to 32 columns, the CUDA-core kernels to the next power of two, the
// few-column kernels run passes of 4 or 8).
constexpr int kTuneCounts[] = {1, 2, 4, 8, 16, 32, 64};
constexpr int kNumTuneCounts = sizeof(kTuneCounts) / sizeof(kTuneCounts[0]);

// Times every engine that runs the mixed product of this operator (A x: CUDA
// cores, tensor cores, few-column kernels; A^T x: CUDA cores, few-column) at
// each count of kTuneCounts, `reps` timed products after one untimed, the
// median kept; the fastest fills h->tuned.  The inputs are one constant (every
// byte 0x3F: 4.8e-4; no kernel branches on values).  The forced engine
// (hodlr3d_set_engine) is restored.
int autotune(hodlr3d_t h, int reps, std::string& report) {
  std::memset(h->tuned, 0, sizeof h->tuned);
  h->tc_split = 0;
  report.clear();
  if (reps == 0) return HODLR3D_OK;
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!h->opt.keep_fp32) return set_error(HODLR3D_ERR_INVALID_ARG, "the mixed form needs keep_fp32");
  const int64_t N = h->N;
  const size_t bytes = sizeof(double) * N * 64;
  DevBuf X, Y;
  H3D_CUDA(X.ensure(bytes));
  H3D_CUDA(Y.ensure(bytes));
  cudaStream_t s = h->stream;
  H3D_CUDA(cudaMemsetAsync(X.p, 0x3F, bytes, s));
  EventPair ev;
  H3D_CUDA(cudaEventCreate(&ev.a));
  H3D_CUDA(cudaEventCreate(&ev.b));
  const int forced = h->engine;
  int8_t choice[2][kNumTuneCounts] = {};
  char line[160];
  report = "transpose nrhs engine ms\n";
  int st = HODLR3D_OK;
  bool tc_runs = false;
  // median of `reps` timed products (after one untimed) under the current
  // engine and launch shapes
  auto time_product = [&](int nrhs, bool tr, float& med) -> int {
    int e2 = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr);
    if (e2 != HODLR3D_OK) return e2;
    std::vector<float> ms(reps);
    for (int r = 0; r < reps; ++r) {
      cudaError_t e = cudaEventRecord(ev.a, s);
      if (e == cudaSuccess) {
        e2 = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr);
        if (e2 != HODLR3D_OK) return e2;
        e = cudaEventRecord(ev.b, s);
      }
      if (e == cudaSuccess) e = cudaEventSynchronize(ev.b);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[r], ev.a, ev.b);
      if (e != cudaSuccess) return set_error(HODLR3D_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(e));
    }
    std::sort(ms.begin(), ms.end());
    med = ms[reps / 2];
    return HODLR3D_OK;
  };
  for (int tr = 0; tr < 2 && st == HODLR3D_OK; ++tr) {
    for (int ci = 0; ci < kNumTuneCounts && st == HODLR3D_OK; ++ci) {
      const int nrhs = kTuneCounts[ci];
      float best = 0.f;
      for (int eng = 1; eng <= 3; ++eng) {
        if (tr && eng == 2) continue;  // no tensor-core transpose
        h->engine = eng;
        // untimed product: builds the engine's tables and buffers
        st = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr != 0);
        if (st == HODLR3D_ERR_UNSUPPORTED) {  // this tree does not suit the engine
          st = HODLR3D_OK;
          continue;
        }
        if (st != HODLR3D_OK) break;
        std::vector<float> ms(reps);
        for (int r = 0; r < reps && st == HODLR3D_OK; ++r) {
          cudaError_t e = cudaEventRecord(ev.a, s);
          if (e == cudaSuccess) {
            st = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr != 0);
            e = cudaEventRecord(ev.b, s);
          }
          if (e == cudaSuccess) e = cudaEventSynchronize(ev.b);
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[r], ev.a, ev.b);
          if (e != cudaSuccess && st == HODLR3D_OK)
            st = set_error(HODLR3D_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(e));
        }
        if (st != HODLR3D_OK) break;
        if (eng == 2) tc_runs = true;
        std::sort(ms.begin(), ms.end());
        const float med = ms[reps / 2];
        std::snprintf(line, sizeof line, "%d %d %d %.6f\n", tr, nrhs, eng, med);
        report += line;
        if (choice[tr][ci] == 0 || med < best) {
          choice[tr][ci] = (int8_t)eng;
          best = med;
        }
      }
    }
  }
  // launch shapes: blocks per slice of the tensor-core T kernel (which tile
  // each block multiplies; the results do not depend on it), 32 columns
  if (st == HODLR3D_OK && tc_runs) {
    h->engine = 2;
    int best_split = 0;
    float best = 0.f;
    std::string lines;
    for (int k : {1, 2, 4, 8, 16, 32}) {
      h->tc_split = k;
      float med = 0.f;
      st = time_product(32, false, med);
      if (st != HODLR3D_OK) break;
      std::snprintf(line, sizeof line, "launch ta_split %d %.6f\n", k, med);
      lines += line;
      if (best_split == 0 || med < best) {
        best_split = k;
        best = med;
      }
    }
    h->tc_split = st == HODLR3D_OK ? best_split : 0;
    report += lines;
    if (st == HODLR3D_OK) {
      std::snprintf(line, sizeof line, "launch ta_split_chosen %d %.6f\n", best_split, best);
      report += line;
    }
  }
  h->engine = forced;
  if (st != HODLR3D_OK) return st;
  for (int tr = 0; tr < 2; ++tr) {
    int ci = 0;
    for (int n = 1; n <= 64; ++n) {
      while (kTuneCounts[ci] < n) ++ci;
      h->tuned[tr][n] = choice[tr][ci];
    }
  }
  return HODLR3D_OK;
}

}  // namespace hodlr3d_host
