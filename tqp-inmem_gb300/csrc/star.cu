// star.cu - fused multi-way star join + group-by + top-k.
//
// Plan shape (main.py executes it as Filter(A), Join(F,A), Join(.,B),
// Join(.,C), Aggregate, take ordered): fact F with foreign keys into
// dimension A (filtered) and dimension B; B carries a foreign key into C;
// group by the C key with sum(expr) and count(*), top-k by the sum.
//
// Every join is on a dimension's primary key, so each dimension becomes a
// direct-address directory over its key domain (a table statistic):
//   A: dir_a[key - min] = 1 when the A row passes its predicate
//   B: dir_b[key - min] = the row's C foreign key (the payload of the next hop)
//   C: dir_c[key - min] = 1 (existence)
// and the fact side is one pass: each row walks A -> B -> C with three
// L2-resident lookups (price/discount are loaded only for the ~20% of rows
// that survive the A filter), and updates the C group's FP64 sum and count
// with L2 atomics.  The groups come out as slots of dir_c, so the top-k of
// the sums (ties by ascending C key, the reference's aggregate order) is the
// warp-list top-k over the slot table.  A repeated dimension key or a key
// outside its stated domain is reported through the workspace error word.
#include <algorithm>

#include "topk.cuh"

namespace tqpk {

struct StarArgs {
  const void* f_fka; int f_fka_dt;
  const void* f_fkb; int f_fkb_dt;
  int64_t nf;
  const void* a_key; int a_dt; int64_t na; int64_t a_min, a_slots;
  const void* b_key; int b_dt; const void* b_fkc; int b_fkc_dt; int64_t nb; int64_t b_min, b_slots;
  const void* c_key; int c_dt; int64_t nc; int64_t c_min, c_slots;
  int val_reg;
  int a_pvec, f_pvec, v_pvec;
};

// Dimension builds: mode 0 = A (predicate -> 1), 1 = B (payload fkc), 2 = C (existence).
__global__ void __launch_bounds__(kBlock) k_star_build(const __grid_constant__ tqpk_predicate P, int mode,
                                                       const void* keys, int dt, const void* payload, int pdt,
                                                       int64_t n, int64_t kmin, int64_t slots, int pvec,
                                                       int* __restrict__ dir, int* err) {
  const int64_t groups = (n + 3) >> 2;
  const bool kvec = ((reinterpret_cast<uintptr_t>(keys) & 15u) == 0);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    uint32_t b = (P.n_insn && mode == 0) ? eval_pred4(P, r0, n, pvec) : (n - r0 >= 4 ? 0xfu : ((1u << (n - r0)) - 1));
    int64_t x[4];
    ld4_int(keys, dt, r0, n, kvec, x);
    int64_t pl[4] = {1, 1, 1, 1};
    if (mode == 1) ld4_int(payload, pdt, r0, n, false, pl);
    int old[4];           // the four claims in flight together, their results read afterwards
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t slot = x[j] - kmin;
      const bool in = r0 + j < n, put = in && slot >= 0 && slot < slots;
      if (in && !put) set_error(err, TQPK_EINVAL);
      // every dimension row claims its key (duplicates are errors); A rows failing
      // the predicate store 0 so the fact probe drops them
      // a payload outside int32 cannot name a C key (the C domain is int32): out-of-domain marker
      const int v = (mode == 0) ? (int)((b >> j) & 1u)
                                : ((pl[j] <= (int64_t)INT32_MIN + 1 || pl[j] > INT32_MAX) ? INT32_MIN + 1 : (int)pl[j]);
      old[j] = put ? atomicCAS(&dir[slot], INT32_MIN, v) : INT32_MIN;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (old[j] != INT32_MIN) set_error(err, TQPK_EUNSUPPORTED);
  }
}

__global__ void __launch_bounds__(kBlock) k_star_probe(const __grid_constant__ tqpk_predicate P,
                                                       const __grid_constant__ tqpk_groupby_spec S, StarArgs A,
                                                       const int* __restrict__ dir_a, const int* __restrict__ dir_b,
                                                       const int* __restrict__ dir_c, double* __restrict__ sum,
                                                       unsigned* __restrict__ cnt,
                                                       unsigned long long* __restrict__ groups) {
  // Two 4-row groups per thread per iteration; each hop (A, B, C) issues the
  // lookups of all surviving rows before the next hop uses them.
  constexpr int U = 2;
  const int64_t n8 = (A.nf + 4 * U - 1) / (4 * U);
  const bool va = ((reinterpret_cast<uintptr_t>(A.f_fka) & 15u) == 0);
  const bool vb = ((reinterpret_cast<uintptr_t>(A.f_fkb) & 15u) == 0);
  const bool tile = tile_ok(S);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n8; g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m[U];
    int64_t k[U][4];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t r0 = (g * U + u) << 2;
      m[u] = P.n_insn ? eval_pred4(P, r0, A.nf, A.f_pvec)
                      : (A.nf - r0 >= 4 ? 0xfu : (A.nf - r0 <= 0 ? 0u : ((1u << (A.nf - r0)) - 1)));
      if (m[u]) ld4_int(A.f_fka, A.f_fka_dt, r0, A.nf, va, k[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t sa = k[u][j] - A.a_min;
        const bool ok = ((m[u] >> j) & 1u) && sa >= 0 && sa < A.a_slots;
        if (!ok || __ldg(&dir_a[sa]) <= 0) m[u] &= ~(1u << j);
      }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (m[u]) ld4_int(A.f_fkb, A.f_fkb_dt, (g * U + u) << 2, A.nf, vb, k[u]);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t sb = k[u][j] - A.b_min;
        const bool ok = ((m[u] >> j) & 1u) && sb >= 0 && sb < A.b_slots;
        const int fkc = ok ? __ldg(&dir_b[sb]) : INT32_MIN;
        if (fkc == INT32_MIN) m[u] &= ~(1u << j);
        k[u][j] = (int64_t)fkc - A.c_min;
      }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t sc = k[u][j];
        const bool ok = ((m[u] >> j) & 1u) && sc >= 0 && sc < A.c_slots;
        if (!ok || __ldg(&dir_c[sc]) == INT32_MIN) m[u] &= ~(1u << j);
      }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!m[u]) continue;
      const int64_t r0 = (g * U + u) << 2;
      double v[4];
      if (tile) {
        ColTile4 T;
        load_cols4(S, r0, A.nf, A.v_pvec != 0, T);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint64_t r[16];
          expr_eval_tile<16>(S.expr, A.val_reg + 1, S.col_dtypes, T, j, r);
          const uint64_t raw = reg_pick<16>(r, A.val_reg);
          v[j] = S.expr[A.val_reg].type == TQPK_F64 ? u2d(raw) : (double)(int64_t)raw;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = ((m[u] >> j) & 1u) ? expr_value(S, r0 + j, A.val_reg) : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!((m[u] >> j) & 1u)) continue;
        gred_add(&sum[k[u][j]], v[j]);
        gred_add(&cnt[k[u][j]], 1u);
      }
    }
  }
}

__global__ void k_star_emit(const int64_t* idx, const int64_t* count, const double* sum, const unsigned* cnt,
                            int64_t key_min, int k, int64_t* out_keys, double* out_vals, int64_t* out_cnts,
                            int64_t* out_count) {
  const int64_t m = *count;
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    if (j < m) {
      out_keys[j] = key_min + idx[j];
      out_vals[j] = sum[idx[j]];
      if (out_cnts) out_cnts[j] = cnt[idx[j]];
    }
  }
  if (threadIdx.x == 0) *out_count = m;
}

constexpr int kStarMaxK = 256;

__global__ void k_fill_i32(int* p, int64_t n, int v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

struct StarLayout {
  int *dir_a, *dir_b, *dir_c;
  double* sum;
  unsigned* cnt;
  unsigned long long* groups;
  int* err;
  unsigned* ticket;
  int64_t* top_count;
  int64_t* top_idx;
  uint64_t* cand_key;
  int64_t* cand_idx;
};

static size_t star_bytes(int64_t as, int64_t bs, int64_t cs, int grid) {
  return 4096 + align_up(as * 4, 256) + align_up(bs * 4, 256) + align_up(cs * 4, 256) + align_up(cs * 8, 256) +
         align_up(cs * 4, 256) + align_up(kStarMaxK * 8, 256) +
         2 * align_up(std::max<size_t>((size_t)grid * kStarMaxK, kTopkCand) * 8, 256);
}

static bool star_layout(void* ws, size_t bytes, int64_t as, int64_t bs, int64_t cs, int grid, StarLayout& L) {
  WsCursor c(ws, bytes);
  int* hdr = c.take<int>(64);
  if (!hdr) return false;
  L.groups = reinterpret_cast<unsigned long long*>(hdr);
  L.err = hdr + 2;
  L.ticket = reinterpret_cast<unsigned*>(hdr + 3);
  L.top_count = reinterpret_cast<int64_t*>(hdr + 4);
  L.dir_a = c.take<int>(as);
  L.dir_b = c.take<int>(bs);
  L.dir_c = c.take<int>(cs);
  L.sum = c.take<double>(cs);
  L.cnt = c.take<unsigned>(cs);
  L.top_idx = c.take<int64_t>(kStarMaxK);
  L.cand_key = c.take<uint64_t>(std::max<size_t>((size_t)grid * kStarMaxK, kTopkCand));
  L.cand_idx = c.take<int64_t>(std::max<size_t>((size_t)grid * kStarMaxK, kTopkCand));
  return L.cand_idx != nullptr;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_pipeline_star_workspace_bytes(int64_t a_slots, int64_t b_slots, int64_t c_slots) {
  return star_bytes(std::max<int64_t>(a_slots, 1), std::max<int64_t>(b_slots, 1), std::max<int64_t>(c_slots, 1),
                    topk_grid_size());
}

extern "C" int tqpk_pipeline_star_agg_topk(
    const void* d_f_fka, int32_t f_fka_dtype, const void* d_f_fkb, int32_t f_fkb_dtype, int64_t nf,
    const tqpk_predicate* h_fact_pred, const tqpk_groupby_spec* h_values, int32_t value_reg,
    const void* d_a_key, int32_t a_dtype, int64_t na, const tqpk_predicate* h_a_pred, int64_t a_min, int64_t a_max,
    const void* d_b_key, int32_t b_dtype, const void* d_b_fkc, int32_t b_fkc_dtype, int64_t nb, int64_t b_min,
    int64_t b_max, const void* d_c_key, int32_t c_dtype, int64_t nc, int64_t c_min, int64_t c_max, int32_t k,
    int32_t descending, void* d_ws, size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_counts,
    int64_t* d_out_count, int64_t* d_groups_out, tqpk_stream stream) {
  if (nf < 0 || na < 0 || nb < 0 || nc < 0 || k < 1 || k > kStarMaxK || !h_values || !d_ws || !d_out_keys ||
      !d_out_vals || !d_out_count)
    return TQPK_EINVAL;
  if ((nf && (!d_f_fka || !d_f_fkb)) || (na && !d_a_key) || (nb && (!d_b_key || !d_b_fkc)) || (nc && !d_c_key))
    return TQPK_EINVAL;
  for (int dt : {f_fka_dtype, f_fkb_dtype, a_dtype, b_dtype, b_fkc_dtype, c_dtype})
    if (!is_int_dtype(dt)) return TQPK_EDTYPE;
  if (a_max < a_min || b_max < b_min || c_max < c_min) return TQPK_EINVAL;
  if (c_min <= (int64_t)INT32_MIN + 1 || c_max > INT32_MAX) return TQPK_EUNSUPPORTED;  // C keys travel as int32
  const int64_t as = a_max - a_min + 1, bs = b_max - b_min + 1, cs = c_max - c_min + 1;
  if (as > (int64_t(1) << 31) || bs > (int64_t(1) << 31) || cs > (int64_t(1) << 31)) return TQPK_EUNSUPPORTED;
  if (value_reg < 0 || value_reg >= h_values->n_expr) return TQPK_EINVAL;
  int rc = nf > 0 ? check_pred(h_fact_pred) : TQPK_OK;   // empty sides never evaluate their predicate
  if (!rc && na > 0) rc = check_pred(h_a_pred);
  if (rc) return rc;
  const int grid = topk_grid_size();
  if (ws_bytes < star_bytes(as, bs, cs, grid)) return TQPK_ENOMEM;
  StarLayout L;
  if (!star_layout(d_ws, ws_bytes, as, bs, cs, grid, L)) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  StarArgs A{d_f_fka, f_fka_dtype, d_f_fkb, f_fkb_dtype, nf, d_a_key, a_dtype, na, a_min, as,
             d_b_key, b_dtype, d_b_fkc, b_fkc_dtype, nb, b_min, bs, d_c_key, c_dtype, nc, c_min, cs,
             value_reg, pred_vec_ok(h_a_pred) ? 1 : 0, pred_vec_ok(h_fact_pred) ? 1 : 0,
             spec_cols_vec(h_values) ? 1 : 0};
  TQPK_CUDA(cudaMemsetAsync(L.groups, 0, 64, s));
  k_fill_i32<<<grid_for(as, 4), kBlock, 0, s>>>(L.dir_a, as, INT32_MIN);
  TQPK_CHECK_LAUNCH();
  k_fill_i32<<<grid_for(bs, 4), kBlock, 0, s>>>(L.dir_b, bs, INT32_MIN);
  TQPK_CHECK_LAUNCH();
  k_fill_i32<<<grid_for(cs, 4), kBlock, 0, s>>>(L.dir_c, cs, INT32_MIN);
  TQPK_CHECK_LAUNCH();
  TQPK_CUDA(cudaMemsetAsync(L.sum, 0, cs * 8, s));
  TQPK_CUDA(cudaMemsetAsync(L.cnt, 0, cs * 4, s));
  const tqpk_predicate& none = *pred_or_empty(nullptr);
  if (na) {
    k_star_build<<<grid_for((na + 3) / 4, 4), kBlock, 0, s>>>(*pred_or_empty(h_a_pred), 0, d_a_key, a_dtype, nullptr,
                                                             0, na, a_min, as, A.a_pvec, L.dir_a, L.err);
    TQPK_CHECK_LAUNCH();
  }
  if (nb) {
    k_star_build<<<grid_for((nb + 3) / 4, 4), kBlock, 0, s>>>(none, 1, d_b_key, b_dtype, d_b_fkc, b_fkc_dtype, nb,
                                                             b_min, bs, 0, L.dir_b, L.err);
    TQPK_CHECK_LAUNCH();
  }
  if (nc) {
    k_star_build<<<grid_for((nc + 3) / 4, 4), kBlock, 0, s>>>(none, 2, d_c_key, c_dtype, nullptr, 0, nc, c_min, cs, 0,
                                                             L.dir_c, L.err);
    TQPK_CHECK_LAUNCH();
  }
  if (nf) {
    timing_before(KID_STAR_PROBE, s);
    k_star_probe<<<occ_grid(k_star_probe, (nf + 7) / 8), kBlock, 0, s>>>(*pred_or_empty(h_fact_pred), *h_values, A,
                                                                       L.dir_a, L.dir_b, L.dir_c, L.sum, L.cnt,
                                                                       L.groups);
    timing_after(KID_STAR_PROBE, s);
    TQPK_CHECK_LAUNCH();
  }
  DenseSumSource src{L.sum, L.cnt, cs, descending ? 1 : 0};
  TopkOut O{L.top_idx, L.top_count, L.cand_key, L.cand_idx, L.ticket, L.groups,
            reinterpret_cast<unsigned long long*>(L.top_count + 1),    // zeroed with the header
            reinterpret_cast<unsigned*>(L.top_count + 2)};
  O.err = L.err;                       // the single-launch top-k (k <= 32) reports a barrier timeout here
  rc = topk_warp_launch(0, &src, k, grid, O, s);
  if (rc) return rc;
  k_star_emit<<<1, 256, 0, s>>>(L.top_idx, L.top_count, L.sum, L.cnt, c_min, k, d_out_keys, d_out_vals, d_out_counts,
                                d_out_count);
  TQPK_CHECK_LAUNCH();
  if (d_groups_out) TQPK_CUDA(cudaMemcpyAsync(d_groups_out, L.groups, 8, cudaMemcpyDeviceToDevice, s));
  return TQPK_OK;
}
