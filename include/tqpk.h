/*
 * tqpk.h - C ABI of libtqpk.so, the GB300 (sm_103a) kernels behind TQP-Inmem's
 * relational operator hot path.
 *
 * Every pointer named d_* or passed inside a column descriptor is a device
 * pointer; h_* pointers are host pointers.  Every entry point returns an int
 * status (TQPK_OK = 0, negative on error) and enqueues its work on the given
 * CUDA stream.  Entry points whose contract says "synchronises" wait on that
 * stream before returning (they need a device-side count on the host, as the
 * reference does with .item()/nonzero at the same places).
 *
 * Reference interfaces replaced (paths inside TQP-Inmem):
 *   tqpk_filter_mask        operators/filter.py:14-162 (evaluate), :164-204 (tqp_filter)
 *   tqpk_compact            IO/vortex_pipeline.py:51-66 (tensor[mask] late materialisation)
 *   tqpk_groupby_*          operators/aggregate.py:236-393 (tqp_hash_aggregate / agg_wrapper / evaluate)
 *   tqpk_argsort_stable     operators/sort.py:22-35 (LSD sequence of stable torch.sort)
 *   tqpk_topk_stable        operators/sort.py:41-42 (full sort, then perm[:limit])
 *   tqpk_join_*             operators/hashjoin.py:24-177 (join_kernel_new), :179-248 (join_vortex)
 *   tqpk_gather             hashjoin.py:153-175 + conversion.py:52-57 (x[idx], index_with_null)
 *   tqpk_pipeline_*         fused forms of filter -> join -> aggregate (main.py:152-253 call order)
 */
#ifndef TQPK_H
#define TQPK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* tqpk_stream; /* a cudaStream_t */

/* ---- status codes ------------------------------------------------------ */
enum {
  TQPK_OK = 0,
  TQPK_EINVAL = -1,       /* bad argument (null pointer, size, count)              */
  TQPK_ENOMEM = -2,       /* workspace too small                                   */
  TQPK_ETIMEOUT = -3,     /* a bounded device-side wait gave up                    */
  TQPK_EDTYPE = -4,       /* unsupported dtype code                                */
  TQPK_ECUDA = -5,        /* CUDA launch/runtime error                             */
  TQPK_ECAPACITY = -6,    /* output capacity too small (required size returned)    */
  TQPK_EUNSUPPORTED = -7  /* shape the kernels do not handle (caller must not fall back) */
};

/* ---- dtype codes (constants.py:3-6: string int8, int int64, float f64, date int32)
 * TQPK_ROWID is accepted only as a tqpk_compact output: it writes each kept
 * row's index (int64) and ignores the input pointer.                        */
enum { TQPK_ROWID = 0, TQPK_I8 = 1, TQPK_U8 = 2, TQPK_I32 = 3, TQPK_I64 = 4, TQPK_F64 = 5, TQPK_BOOL = 6 };

#define TQPK_MAX_COLS 16
#define TQPK_MAX_PRED 32
#define TQPK_MAX_KEYS 4
#define TQPK_MAX_EXPR 32
#define TQPK_MAX_ACCS 16
#define TQPK_NULL_INDEX (-64) /* constants.py:9 null, used by index_with_null */

/* ---- predicate program (filter.py:14-162) --------------------------------
 * Postfix program over up to TQPK_MAX_COLS columns.  CMP pushes
 * (col <cmp> literal) evaluated in `domain`; AND/OR pop two, NOT pops one;
 * TRUE pushes all-true (isnotnull, filter.py:67-69); MASK pushes a bool column.
 *   domain I64: integer column vs Python int, exact.
 *   domain F64: float64 column (or int column vs int literal on a float column).
 *   domain F32: integer column vs Python float (torch promotes to float32).
 *   ISCLOSE: |x - lit| <= lit_aux (allowed error, precomputed as atol + |rtol*lit|)
 *            or x == lit, as torch.isclose (filter.py:160-161).
 * Float literals for <= and >= arrive with the reference's +-eps already added
 * (filter.py:145-149).                                                      */
enum { TQPK_P_CMP = 1, TQPK_P_AND = 2, TQPK_P_OR = 3, TQPK_P_NOT = 4, TQPK_P_TRUE = 5,
       TQPK_P_FALSE = 6, TQPK_P_MASK = 7, TQPK_P_CMPCOL = 8 /* cols[col] <cmp> cols[lit_i] */,
       /* string columns: int8 [N, w], w = widths[col]; literals are bytes of strpool.
        * STRCMP: every byte of the row <cmp> the literal padded to w (lit_i = offset),
        *         the reference's multi-character comparison (filter.py:151-158).
        * PREFIX: the first len bytes equal the literal (StartsWith, filter.py:48-55).
        * CONTAINS: the literal occurs at some position (Contains/EndsWith, like.py:3-11).
        *         PREFIX/CONTAINS: lit_i = offset | len << 32.
        * LIKE2:  '%a%b%': b starts at or after the end of an occurrence of a (like.py:13-22);
        *         lit_i = off_a | len_a << 16 | off_b << 32 | len_b << 48.            */
       TQPK_P_STRCMP = 9, TQPK_P_PREFIX = 10, TQPK_P_CONTAINS = 11, TQPK_P_LIKE2 = 12 };
enum { TQPK_LT = 0, TQPK_LE = 1, TQPK_GT = 2, TQPK_GE = 3, TQPK_EQ = 4, TQPK_NE = 5, TQPK_ISCLOSE = 6 };
enum { TQPK_DOM_I64 = 0, TQPK_DOM_F64 = 1, TQPK_DOM_F32 = 2 };

typedef struct {
  int32_t op, col, cmp, domain;
  int64_t lit_i;
  double lit_f;
  double lit_aux;
} tqpk_pred_insn;

#define TQPK_MAX_STRPOOL 512

typedef struct {
  int32_t n_insn;
  int32_t n_cols;
  const void* cols[TQPK_MAX_COLS];
  int32_t dtypes[TQPK_MAX_COLS];
  tqpk_pred_insn insn[TQPK_MAX_PRED];
  int32_t widths[TQPK_MAX_COLS];      /* bytes per row of an int8 [N, w] string column, else 0 */
  uint8_t strpool[TQPK_MAX_STRPOOL];  /* literal bytes of the string instructions */
  int32_t strides[TQPK_MAX_COLS];     /* row stride of a string column view (substring, filter.py:71-76):
                                         bytes between rows; 0 = the width */
} tqpk_predicate;

/* ---- row expressions (aggregate.py:58-233) --------------------------------
 * Straight-line SSA program: instruction i writes register i.  Operands a, b
 * are earlier register numbers.  Arithmetic follows torch's promotion:
 * registers are float64 or int64 (`type`); float64 arithmetic is IEEE
 * round-to-nearest per operation (no contraction), as torch evaluates it.
 * A register of type TQPK_F32 (registers only; no column has it) holds a
 * float32 in its low 32 bits: torch's result for an integer tensor with a
 * Python float, an integer true division or a CASE mixing a float literal
 * with integers (torch's default float dtype), computed in float32 with
 * round-to-nearest.  TQPK_X_TOF32 converts an int64 register to float32,
 * TQPK_X_F32TOF64 a float32 register to float64 (exact).
 * TQPK_X_SELECT is torch.where(a != 0, b, col) (CASE WHEN, aggregate.py:76-87;
 * register `col` holds the ELSE value, the condition is a 0/1 register, e.g.
 * a bool column).  TQPK_X_YEAR maps int64 days since 1990-01-01 to the year
 * (aggregate.py:100-101: bucketize over the cumulative year lengths of
 * 1990-1999; days before 1990 give 1990, days from 2000 on the calendar year,
 * where the reference's year table has no entry).                         */
enum { TQPK_X_COL = 1, TQPK_X_CONST = 2, TQPK_X_ADD = 3, TQPK_X_SUB = 4, TQPK_X_MUL = 5,
       TQPK_X_DIV = 6, TQPK_X_TOF64 = 7, TQPK_X_SELECT = 8, TQPK_X_YEAR = 9, TQPK_X_TOF32 = 10,
       TQPK_X_F32TOF64 = 11 };
enum { TQPK_F32 = 7 };   /* expression register type (float32 in the low 32 bits) */

typedef struct {
  int32_t op, type; /* type: TQPK_I64, TQPK_F64 or TQPK_F32 */
  int32_t a, b;     /* operand registers */
  int32_t col;      /* TQPK_X_COL: column slot; TQPK_X_SELECT: ELSE register */
  int32_t wrap;     /* integer ADD/SUB/MUL: 0, or TQPK_I8 / TQPK_U8 / TQPK_I32 when torch's result
                       dtype is that narrower integer: the int64 result is wrapped to it (two's
                       complement), as torch's int8 / uint8 / int32 arithmetic wraps */
  int64_t ci;       /* TQPK_X_CONST integer value */
  double cf;        /* TQPK_X_CONST float value */
} tqpk_expr_insn;

/* Accumulators (aggregate.py:122-195).  sum/avg/count/min/max of the
 * reference map onto these; avg = SUM / COUNT_ROWS at emit.
 * MAX starts from 0 and MIN from the dtype maximum, as the reference's
 * scatter_reduce initial tensors do (aggregate.py:154-167).               */
enum { TQPK_ACC_SUM = 1, TQPK_ACC_COUNT_NOTNULL = 2, TQPK_ACC_COUNT_ROWS = 3, TQPK_ACC_MIN = 4,
       TQPK_ACC_MAX = 5 };

typedef struct {
  int32_t kind;  /* TQPK_ACC_* */
  int32_t type;  /* TQPK_F64 or TQPK_I64: register type of `reg` */
  int32_t reg;   /* expression register accumulated (ignored by COUNT_ROWS) */
  int32_t pad;
  int64_t init_i; /* MIN/MAX initial value for I64 */
  double init_f;  /* MIN/MAX initial value for F64 */
} tqpk_acc;

typedef struct {
  int32_t n_keys;
  const void* keys[TQPK_MAX_KEYS];
  int32_t key_dtypes[TQPK_MAX_KEYS];
  int32_t n_cols;
  const void* cols[TQPK_MAX_COLS];
  int32_t col_dtypes[TQPK_MAX_COLS];
  int32_t n_expr;
  tqpk_expr_insn expr[TQPK_MAX_EXPR];
  int32_t n_accs;
  tqpk_acc accs[TQPK_MAX_ACCS];
} tqpk_groupby_spec;

/* Plan chosen from the key ranges (tqpk_groupby_plan). */
enum { TQPK_GB_GLOBAL_ONE = 0, TQPK_GB_DENSE_PRIVATE = 1, TQPK_GB_DENSE_SHARED = 2,
       TQPK_GB_DENSE_GLOBAL = 3, TQPK_GB_HASH = 4 };

typedef struct {
  int32_t mode;
  int32_t threads;
  int64_t n_rows;                /* rows passing the filter */
  int64_t slots;                 /* dense slots or hash capacity */
  int64_t key_min[TQPK_MAX_KEYS];
  int64_t key_range[TQPK_MAX_KEYS];
  int64_t key_stride[TQPK_MAX_KEYS];
  size_t ws_bytes;               /* workspace needed by run + emit */
} tqpk_gb_plan;

/* ---- general --------------------------------------------------------- */
int tqpk_version(void);
const char* tqpk_status_string(int status);
/* Number of kernel launches this thread has issued through the library. */
int64_t tqpk_launch_count(void);
/* Writes sizeof() of tqpk_pred_insn, tqpk_predicate, tqpk_expr_insn, tqpk_acc,
 * tqpk_groupby_spec, tqpk_gb_plan, tqpk_join_plan (in that order, up to n of
 * them) so bindings can verify their struct layouts; returns the count.   */
int tqpk_abi_sizes(int64_t* out, int n);

/* Kernel timing (for roofline measurement): after tqpk_timing_begin(id),
 * every launch of kernel `id` is bracketed by CUDA events on its stream;
 * tqpk_timing_end synchronises on them and returns the summed device time.
 * Ids: 1 filter mask, 3 group-by, 5 join probe, 6 fused probe+aggregate,
 * 7 fused build, 8 fused top-k, 9 star-join probe, 10 batched work queue.  */
int tqpk_timing_begin(int32_t kernel_id);
int tqpk_timing_end(double* h_total_ms, int32_t* h_launches);

/* ---- (a) filter -------------------------------------------------------- */
/* mask[i] = pred(row i) for i < n; *d_count += number of true rows.
 * d_count may be NULL.  Replaces filter.py:14-204.                         */
int tqpk_filter_mask(const tqpk_predicate* h_pred, int64_t n, uint8_t* d_mask,
                     unsigned long long* d_count, tqpk_stream stream);

/* Stream compaction, stable: keeps rows where d_mask[i] != 0 (or, when
 * d_mask is NULL, where the predicate holds).  Writes *d_count (int64): the
 * number of rows kept, or a negative status (TQPK_ETIMEOUT) when a bounded
 * device-side wait gave up, in which case the outputs are not valid.
 * Replaces vortex_pipeline.py:58 (tensor[mask]) for up to TQPK_MAX_COLS
 * columns in one pass.                                                    */
size_t tqpk_compact_workspace_bytes(int64_t n);
int tqpk_compact(const tqpk_predicate* h_pred, const uint8_t* d_mask, int64_t n, int32_t ncols,
                 const void* const* h_cols_in, const int32_t* h_dtypes, void* const* h_cols_out,
                 int64_t* d_count, void* d_ws, size_t ws_bytes, tqpk_stream stream);

/* Stream compaction for callers that cannot allocate device memory when
 * they call: an engine that owns all device memory through its own arena, or
 * a serving loop that allows no cudaMalloc after start-up (it can stall the
 * device and can fail mid-request).  No counterpart in the reference, which
 * always allocates through torch.  Same arguments and results as
 * tqpk_compact, minus the workspace.
 * Its scratch is a 1 MiB array inside the library, resident on every device
 * that loads it.  Inputs longer than tqpk_compact_noalloc_max_rows() rows
 * return TQPK_ENOMEM.  All calls on a device share that array, so calls that
 * overlap on the GPU race and must be ordered by the caller.  The first call
 * on a device looks up the array's address; make it before any stream
 * capture on that device.                                                 */
int64_t tqpk_compact_noalloc_max_rows(void);
int tqpk_compact_noalloc(const tqpk_predicate* h_pred, const uint8_t* d_mask, int64_t n, int32_t ncols,
                         const void* const* h_cols_in, const int32_t* h_dtypes, void* const* h_cols_out,
                         int64_t* d_count, tqpk_stream stream);

/* [min, max] of an integer column over its n rows, read to the host (one
 * synchronisation): the key domain a fused join sizes its directory by
 * (hashjoin.py:50-56 sorts the build keys for the same purpose).  d_scratch:
 * 256 bytes.  n == 0 gives min > max.                                     */
int tqpk_key_range(const void* d_col, int32_t dtype, int64_t n, void* d_scratch, int64_t* h_min,
                   int64_t* h_max, tqpk_stream stream);

/* Test hook, no counterpart in the reference: the poll limit of the
 * compaction's look-back (<= its default) and a tile whose CTA publishes
 * nothing (-1: none).  With a tile stalled, its successors' bounded waits run
 * out and the next compactions report TQPK_ETIMEOUT in *d_count.  (2097152, -1)
 * restores the defaults.  Process-wide and not thread-safe.              */
int tqpk_debug_compact_wait(int32_t spin_limit, int64_t stall_tile);

/* Test hook, no counterpart in the reference: the poll limit (<= its
 * default) of the single-launch top-k's grid barrier (k <= 32, the fused
 * pipelines) and a number of arrivals (0-1024) it also waits for that never
 * come.  With missing > 0 every CTA's bounded wait runs out and the pipeline
 * reports TQPK_ETIMEOUT in its error word.  (2097152, 0) restores the
 * defaults.  Process-wide and not thread-safe.                            */
int tqpk_debug_topk_barrier(int32_t spin_limit, int32_t missing);

/* ---- (d) group-by aggregation ----------------------------------------- */
/* Computes the key ranges of the rows passing the filter (d_mask or h_pred,
 * either may be NULL) and picks the kernel.  Synchronises.                */
int tqpk_groupby_plan(const tqpk_groupby_spec* h_spec, const tqpk_predicate* h_pred,
                      const uint8_t* d_mask, int64_t n, tqpk_gb_plan* h_plan,
                      void* d_scratch32, tqpk_stream stream);
/* Accumulates every passing row into the plan's table (filter fused: rows
 * that fail the predicate are never materialised) and counts the groups
 * into *h_groups.  Synchronises.                                          */
int tqpk_groupby_run(const tqpk_groupby_spec* h_spec, const tqpk_gb_plan* h_plan,
                     const tqpk_predicate* h_pred, const uint8_t* d_mask, int64_t n, void* d_ws,
                     size_t ws_bytes, int64_t* h_groups, tqpk_stream stream);
/* Writes the groups in ascending key-tuple order: one column per key (in the
 * key's dtype) and n_out value columns.  h_out_ops holds 4 ints per output:
 * {op, a, b, dtype}: op TQPK_OUT_ACC copies accumulator a; TQPK_OUT_AVG
 * writes acc a / acc b in float64 (aggregate.py:168-177).  dtype is the
 * output column's dtype code.  groups must be the count run returned.      */
enum { TQPK_OUT_ACC = 0, TQPK_OUT_AVG = 1 };
int tqpk_groupby_emit(const tqpk_groupby_spec* h_spec, const tqpk_gb_plan* h_plan, void* d_ws,
                      int64_t groups, void* const* h_out_keys, int32_t n_out, const int32_t* h_out_ops,
                      void* const* h_out_cols, tqpk_stream stream);

/* ---- (b) sort ---------------------------------------------------------- */
/* Stable LSD radix sort of keys[perm_in[i]] (perm_in NULL = identity) with
 * payload perm_in[i]; writes the sorted permutation (int64) to d_perm_out.
 * One call is one iteration of sort.py:26-35's key loop.  descending keeps
 * ties in input order (torch.sort(stable=True, descending=True)).
 * Float keys: -0.0 sorts equal to +0.0 and NaN sorts as the largest value.
 * n <= 2048 sorts in one CTA without a workspace (d_ws may be NULL) and
 * without a host synchronisation; larger sorts synchronise twice.          */
size_t tqpk_sort_workspace_bytes(int64_t n);
int tqpk_argsort_stable(const void* d_keys, int32_t key_dtype, int32_t descending,
                        const int64_t* d_perm_in, int64_t n, int64_t* d_perm_out, void* d_ws,
                        size_t ws_bytes, tqpk_stream stream);

/* ---- (e) top-k ------------------------------------------------------------
 * The first k entries of the stable sort of keys[perm_in[i]]:
 * d_perm_out[0..k) = perm_in of the k smallest (largest if descending) keys,
 * ties in input order.  Equals sort.py:41-42 (full stable sort, then
 * perm[:limit]) without sorting the rest.                                   */
size_t tqpk_topk_workspace_bytes(int64_t n, int64_t k);
int tqpk_topk_stable(const void* d_keys, int32_t key_dtype, int32_t descending,
                     const int64_t* d_perm_in, int64_t n, int64_t k, int64_t* d_perm_out,
                     void* d_ws, size_t ws_bytes, tqpk_stream stream);

/* ---- (c) join ---------------------------------------------------------- */
enum { TQPK_JOIN_DIRECT = 1, TQPK_JOIN_SORTED = 2 };
enum { TQPK_JT_INNER = 0, TQPK_JT_SEMI = 1, TQPK_JT_ANTI = 2, TQPK_JT_OUTER = 3 };

typedef struct {
  int32_t mode;        /* TQPK_JOIN_DIRECT (dense key range) or TQPK_JOIN_SORTED */
  int32_t unique;      /* build keys are unique (set by tqpk_join_build) */
  int64_t nb_rows;     /* build rows passing the build filter */
  int64_t key_min, key_max;
  int64_t slots;       /* DIRECT: key_max - key_min + 1 */
  int64_t n_unique;    /* SORTED: distinct build keys (set by tqpk_join_build) */
  size_t ws_bytes;     /* build workspace (kept alive until the probes are done) */
} tqpk_join_plan;

/* Build-side key range of the rows passing the build mask; picks the mode.
 * Synchronises.                                                            */
int tqpk_join_plan_build(const void* d_build_keys, int32_t key_dtype, const uint8_t* d_build_mask,
                         int64_t nb, tqpk_join_plan* h_plan, void* d_scratch32,
                         tqpk_stream stream);
/* Builds the directory (DIRECT: key -> build row, CSR of rows for duplicate
 * keys; SORTED: radix-sorted (key,row) with run starts).  Synchronises to
 * learn whether the build keys are unique.                                  */
int tqpk_join_build(tqpk_join_plan* h_plan, const void* d_build_keys, int32_t key_dtype,
                    const uint8_t* d_build_mask, int64_t nb, void* d_ws, size_t ws_bytes,
                    tqpk_stream stream);
/* Probes every probe row passing its mask against the directory that
 * tqpk_join_build left in d_build_ws and writes the matches in the
 * reference's order (ascending probe row; inside one build-key bucket,
 * ascending build row) as int64 row ids of the ORIGINAL (uncompacted)
 * inputs.  INNER writes pairs; SEMI/ANTI write probe rows only (d_out_build
 * unused, may be NULL); OUTER writes the pairs, then the unmatched probe rows
 * with build id TQPK_NULL_INDEX.  *h_count is the number of outputs; when it
 * exceeds capacity only the first `capacity` are written and TQPK_ECAPACITY
 * is returned (call again with a larger buffer).  Synchronises.             */
size_t tqpk_join_probe_workspace_bytes(int64_t np);
int tqpk_join_probe(const tqpk_join_plan* h_plan, const void* d_build_ws, const void* d_probe_keys,
                    int32_t probe_dtype, const uint8_t* d_probe_mask, int64_t np, int32_t join_type,
                    int64_t* d_out_build, int64_t* d_out_probe, int64_t capacity, int64_t* h_count,
                    void* d_probe_ws, size_t probe_ws_bytes, tqpk_stream stream);

/* ---- fused pipelines ------------------------------------------------------
 * Filter -> inner join on a unique build key -> sum(expr) group by build key
 * -> top-k by the sum (k <= 256), with no host synchronisation: the main.py
 * plan Filter(build), Filter(probe), Join, Aggregate, take ordered in three
 * kernels.  [key_min, key_max] is the build table's key domain (a table
 * statistic); the directory has one slot per key in it.  h_values holds the
 * expression program over probe columns, value_reg the register summed.
 * d_out_keys/d_out_vals receive min(k, groups) rows ordered by the sum
 * (descending when `descending`), ties by ascending key; *d_out_count that
 * count and *d_groups_out (may be NULL) the number of groups.  A repeated
 * build key or one outside [key_min, key_max] sets the workspace error word
 * (read it with tqpk_pipeline_error: TQPK_EUNSUPPORTED / TQPK_EINVAL); the
 * caller then runs the operator path instead.                              */
size_t tqpk_pipeline_join_agg_topk_workspace_bytes(int64_t key_min, int64_t key_max);
int tqpk_pipeline_join_agg_topk(const void* d_build_keys, int32_t build_dtype, int64_t nb,
                                const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                                const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                                const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                                int32_t value_reg, int32_t k, int32_t descending, void* d_ws, size_t ws_bytes,
                                int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_count,
                                int64_t* d_groups_out, tqpk_stream stream);
/* Star join: fact (fkA, fkB, value columns) joins dimension A (filtered by
 * h_a_pred), dimension B (whose column fkC references C) and dimension C;
 * sum(expr) and count(*) grouped by the C key, top-k by the sum (k <= 256).
 * Every dimension key must be unique (a primary key) inside its stated
 * domain [min, max]; otherwise the workspace error word is set.  Outputs:
 * keys (C key), sums, counts (may be NULL), *d_out_count rows.              */
size_t tqpk_pipeline_star_workspace_bytes(int64_t a_slots, int64_t b_slots, int64_t c_slots);
int tqpk_pipeline_star_agg_topk(const void* d_f_fka, int32_t f_fka_dtype, const void* d_f_fkb, int32_t f_fkb_dtype,
                                int64_t nf, const tqpk_predicate* h_fact_pred, const tqpk_groupby_spec* h_values,
                                int32_t value_reg, const void* d_a_key, int32_t a_dtype, int64_t na,
                                const tqpk_predicate* h_a_pred, int64_t a_min, int64_t a_max, const void* d_b_key,
                                int32_t b_dtype, const void* d_b_fkc, int32_t b_fkc_dtype, int64_t nb,
                                int64_t b_min, int64_t b_max, const void* d_c_key, int32_t c_dtype, int64_t nc,
                                int64_t c_min, int64_t c_max, int32_t k, int32_t descending, void* d_ws,
                                size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_counts,
                                int64_t* d_out_count, int64_t* d_groups_out, tqpk_stream stream);
/* ---- batched instances (one persistent launch) -----------------------------
 * Many independent JOIN-shaped (as tqpk_pipeline_join_agg_topk, k <= 32) and
 * GROUPBY-shaped (filter + dense group-by + ordered emit) instances run as
 * phase-major work items of one persistent kernel fed by an atomic ticket.
 * Each instance is described into an opaque host record of
 * tqpk_batch_record_bytes() bytes (the records are then copied to the device
 * by the caller); rows_per_item / slots_per_item size its work items.  An item
 * of phase p waits (bounded) for the instance's phase p-1 items.  Reset +
 * run only enqueue memsets and kernels on the stream (capturable in a CUDA
 * graph).  Group-by keys use caller-provided domains (table statistics).  */
size_t tqpk_batch_record_bytes(void);
size_t tqpk_batch_join_workspace_bytes(int64_t key_min, int64_t key_max);
int tqpk_batch_describe_join(void* h_rec, const void* d_build_keys, int32_t build_dtype, int64_t nb,
                             const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                             const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                             const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                             int32_t value_reg, int32_t k, int32_t descending, void* d_ws, size_t ws_bytes,
                             int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_count,
                             int64_t* d_groups_out, int64_t build_rows_per_item, int64_t probe_rows_per_item);
size_t tqpk_batch_groupby_workspace_bytes(const tqpk_groupby_spec* h_spec, const int64_t* key_min,
                                          const int64_t* key_max, int64_t slots_per_item);
int tqpk_batch_describe_groupby(void* h_rec, const tqpk_groupby_spec* h_spec, const tqpk_predicate* h_pred,
                                int64_t n, const int64_t* key_min, const int64_t* key_max, void* d_ws,
                                size_t ws_bytes, void* const* h_out_keys, int32_t n_out, const int32_t* h_out_ops,
                                void* const* h_out_cols, int64_t* d_groups_out, int64_t rows_per_item,
                                int64_t slots_per_item, int32_t prefer_private);
/* Writes the phase-major work items (24 bytes each) of n_inst host records;
 * returns the item count (the required count when it exceeds cap).        */
int64_t tqpk_batch_items(const void* h_recs, int32_t n_inst, void* h_items, int64_t cap);
size_t tqpk_batch_ctl_bytes(int32_t n_inst);
int tqpk_batch_reset(const void* h_recs, const void* d_recs, int32_t n_inst, void* d_ctl, tqpk_stream stream);
int tqpk_batch_run(const void* d_recs, int32_t n_inst, const void* d_items, int32_t n_items, void* d_ctl,
                   int32_t grid, tqpk_stream stream);
int tqpk_batch_error(const void* d_ctl, int* h_err, tqpk_stream stream);
int32_t tqpk_batch_grid(void);
/* Per-item timeline (32 bytes per work item: dequeue, dependency met and
 * completion times in ns, SM id) written by later tqpk_batch_run launches
 * while d_trace is set; NULL turns it off.                                  */
int tqpk_batch_set_trace(void* d_trace);

/* ---- runtime-compiled query kernels (NVRTC, opened with dlopen) ----------
 * The host generates CUDA C++ for one query's hot loop (predicate, expression
 * and accumulators as straight-line code); these compile it for sm_103a,
 * load it and launch it.  tqpk_jit_available() is 0 when NVRTC cannot be
 * opened; the interpreting kernels then run instead.                        */
int tqpk_jit_available(void);
int tqpk_jit_check(const char* src, char* log, size_t log_len);
int tqpk_jit_compile(const char* src, const char* name, void** h_handle, char* log, size_t log_len);
int tqpk_jit_occupancy(void* handle, int32_t block, size_t smem);
int tqpk_jit_launch(void* handle, int32_t grid, int32_t block, size_t smem, void** args, int32_t timing_kid,
                    tqpk_stream stream);
/* Preferred shared-memory share of the SM's unified L1/shared storage for a
 * compiled kernel (percent of the maximum, 0-100; a hint the driver rounds
 * to a supported split): a probe that keeps a small lookup structure in L1
 * asks for no more shared memory than its CTAs use.  A launch setting with
 * no counterpart in the reference (its joins run as ATen calls).            */
int tqpk_jit_prefer_shared(void* handle, int32_t percent);
int32_t tqpk_num_sms(void);
/* A group-by plan from key domains known ahead (table statistics [key_min, key_max]
 * per key), with no pass over the data and no host synchronisation; n_rows sizes
 * the hash mode.  The groups still come out only for occupied slots.          */
int tqpk_groupby_plan_domains(const tqpk_groupby_spec* h_spec, const int64_t* h_key_min, const int64_t* h_key_max,
                              int64_t n_rows, tqpk_gb_plan* h_plan);
/* Stages of tqpk_groupby_run around a caller-launched accumulation kernel. */
int tqpk_groupby_prepare(const tqpk_groupby_spec* h_spec, const tqpk_gb_plan* h_plan, void* d_ws, size_t ws_bytes,
                         tqpk_stream stream);
int tqpk_groupby_count(const tqpk_groupby_spec* h_spec, const tqpk_gb_plan* h_plan, void* d_ws, int64_t* h_groups,
                       tqpk_stream stream);
void* tqpk_groupby_table(void* d_ws);
/* The fused join pipeline run stage by stage (bit 0 reset + build, bit 1
 * probe, bit 2 top-k + emit), and the addresses of its tables.  Bit 3 (with
 * a caller-launched probe): the group sums start at -0.0 and carry the
 * occupancy (the probe adds -0.0 values as +0.0 and writes no occupancy
 * word); give it to the reset and the top-k stages alike.  Bit 4 (with a
 * caller-launched probe, not with bit 1): the reset + build stage writes the
 * build side's membership bitmap (bit s of word s / 32 for key key_min + s,
 * (slots + 31) / 32 words at the directory's address) instead of its row
 * directory; a repeated key still sets TQPK_EUNSUPPORTED.  Bit 5 (with bit
 * 4): the reset stage clears the header and the bitmap but launches no build
 * kernel; the caller's build (a query-specialised kernel) sets every group
 * sum to -0.0, the bit of each passing build key (an out-of-domain key sets
 * TQPK_EINVAL in the error word) and adds the passing rows to the count whose
 * address tqpk_pipeline_join_words gives, as the library's build does.      */
int tqpk_pipeline_join_agg_topk_stages(int32_t stages, const void* d_build_keys, int32_t build_dtype, int64_t nb,
                                       const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                                       const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                                       const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                                       int32_t value_reg, int32_t k, int32_t descending, void* d_ws, size_t ws_bytes,
                                       int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_count,
                                       int64_t* d_groups_out, tqpk_stream stream);
int tqpk_pipeline_join_tables(void* d_ws, size_t ws_bytes, int64_t key_min, int64_t key_max, void** dir, void** sum,
                              void** occ);
/* The pipeline's error word and passing-build-row count (uint64), for a caller-launched build. */
int tqpk_pipeline_join_words(void* d_ws, size_t ws_bytes, int64_t key_min, int64_t key_max, int32_t** err,
                             uint64_t** passing);

/* ---- resident directories and dense slot tables (dense.cu) ---------------
 * Replaces the per-call build of operators/hashjoin.py:24-177 (torch.sort of
 * the build keys, then searchsorted) for a join on a unique key: a
 * direct-address directory built once per loaded table and kept in HBM.
 * dir[key - key_min] = payload (the row index when d_payload is NULL) for
 * rows passing h_pred (NULL = all), fail_value for the others, `empty` where
 * no row has the key; a payload outside int32 or equal to `empty` is stored
 * as fail_value.  A key outside [key_min, key_min + slots) sets TQPK_EINVAL
 * in *d_err, a repeated key TQPK_EUNSUPPORTED.                              */
int tqpk_directory_build(const void* d_keys, int32_t key_dtype, int64_t n, const tqpk_predicate* h_pred,
                         const void* d_payload, int32_t payload_dtype, int64_t key_min, int64_t slots, int32_t empty,
                         int32_t fail_value, int32_t* d_dir, int32_t* d_err, tqpk_stream stream);
/* Snowflake chain B -> C: an entry of d_dir that names a key of the next
 * table's domain (B's directory holding C keys) keeps it only when the next
 * directory has a row at that key (d_next[v - next_min] >= 0, e.g. C's row
 * directory with C's filter applied), else becomes fail_value; a probe through
 * the composed directory then needs no lookup in the next one.              */
int tqpk_directory_compose(int32_t* d_dir, int64_t slots, const int32_t* d_next, int64_t next_min,
                           int64_t next_slots, int32_t empty, int32_t fail_value, tqpk_stream stream);
/* tqpk_directory_build with the composition built in: a payload (a key of
 * the next table's domain) is kept only when d_next[payload - next_min] >= 0,
 * else the entry becomes fail_value; the same directory as build followed by
 * tqpk_directory_compose, without the second pass over it.  d_next is built
 * first (the snowflake chain's last table first).  Replaces, for a chain of
 * inner joins on primary keys, the build side of two successive join_vortex
 * calls (operators/hashjoin.py:179-248, main.py:198-244).                  */
int tqpk_directory_build_next(const void* d_keys, int32_t key_dtype, int64_t n, const tqpk_predicate* h_pred,
                              const void* d_payload, int32_t payload_dtype, int64_t key_min, int64_t slots,
                              int32_t empty, int32_t fail_value, const int32_t* d_next, int64_t next_min,
                              int64_t next_slots, int32_t* d_dir, int32_t* d_err, tqpk_stream stream);
/* Membership bitmap of a row directory: bit s of d_bits (word s / 32, bit
 * s % 32) is set when d_dir[s] >= 0.  d_bits holds (slots + 31) / 32 words.
 * A probe that only asks whether a dimension key has a row that passed the
 * dimension's filter (the star join's A table, filtered at build) reads
 * 1 bit per key instead of 4 bytes, so its lookups stay in L1/L2; the same
 * membership test as the reference's inner join on a unique, pre-filtered
 * build side (operators/hashjoin.py:24-177 with the filter of
 * operators/filter.py:164-204 applied first).                               */
int tqpk_directory_bits(const int32_t* d_dir, int64_t slots, uint32_t* d_bits, tqpk_stream stream);
/* The k (<= 256) best groups of a dense slot table (sum[s], count[s] != 0
 * marks a group) ordered by sum (descending when `descending`), ties to the
 * smaller key: the "sort by aggregate + limit" of operators/sort.py:6-58 over
 * a group-by result in ascending key order (aggregate.py:325 unique order).
 * Keys are key_min + slot.  No host synchronisation.                       */
size_t tqpk_dense_topk_workspace_bytes(int32_t k);
int tqpk_dense_topk(const double* d_sum, const uint32_t* d_cnt, int64_t slots, int64_t key_min, int32_t k,
                    int32_t descending, void* d_ws, size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals,
                    int64_t* d_out_counts, int64_t* d_out_count, int64_t* d_out_groups, tqpk_stream stream);
/* tqpk_groupby_emit without the host synchronisation: outputs hold
 * h_plan->slots rows; *d_groups_out receives the group count (or a negative
 * status).                                                                   */
int tqpk_groupby_emit_async(const tqpk_groupby_spec* h_spec, const tqpk_gb_plan* h_plan, void* d_ws,
                            void* const* h_out_keys, int32_t n_out, const int32_t* h_out_ops,
                            void* const* h_out_cols, int64_t* d_groups_out, tqpk_stream stream);

/* Reads (synchronising) the error word a fused pipeline left in its workspace. */
int tqpk_pipeline_error(const void* d_ws, int* h_err, tqpk_stream stream);

/* flags[idx[j]] = 1 for each j (indices outside [0, n) skipped): the probe rows
 * that keep a pair after a join's extra conditions, from which the semi, anti
 * and outer forms are compacted (hashjoin.py:110-151).                       */
int tqpk_mark_rows(const int64_t* d_idx, int64_t n_idx, uint8_t* d_flags, int64_t n, tqpk_stream stream);

/* Multi-column gather: out_c[j] = in_c[idx[j]]; with null_aware, an index
 * equal to TQPK_NULL_INDEX gives the value -64 (conversion.py:52-57).       */
int tqpk_gather(int32_t ncols, const void* const* h_cols_in, const int32_t* h_dtypes,
                const int64_t* d_idx, int64_t n_idx, int32_t null_aware, void* const* h_cols_out,
                tqpk_stream stream);

/* ---- group codes of arbitrary key tuples (aggregate.py:291-333) ----------
 * Key tuples of up to TQPK_MAX_COLS columns: 1-D integer or float64 keys
 * (h_widths[k] = 0) and int8/uint8 [N, w] string keys (h_widths[k] = w), the
 * columns the reference stacks side by side before numbering the distinct
 * rows.  Rows passing d_mask (NULL = all) get d_codes[r] in [0, G), ordered by
 * key tuple ascending (numbers by value, float64 -0.0 == +0.0, strings byte by
 * byte as int8); masked rows get 0.  d_reps[g] (room for n) is a row of group
 * g.  Synchronises once (for G).                                            */
size_t tqpk_key_encode_workspace_bytes(int64_t n);
int tqpk_key_encode(int32_t n_keys, const void* const* h_keys, const int32_t* h_dtypes, const int32_t* h_widths,
                    const uint8_t* d_mask, int64_t n, int32_t* d_codes, int64_t* d_reps, int64_t* h_groups,
                    void* d_ws, size_t ws_bytes, tqpk_stream stream);

/* Row gather of fixed-width rows (a 2-D [N, w] column): dst[j] = src[idx[j]],
 * row_bytes bytes each (hashjoin.py:153-175 and aggregate.py:323-325 for
 * string columns).  Indices outside [0, n_src) give zero rows.               */
int tqpk_gather_rows(const void* d_src, int64_t n_src, int64_t row_bytes, const int64_t* d_idx, int64_t n_idx,
                     void* d_dst, tqpk_stream stream);

/* Sort keys of a string column for tqpk_argsort_stable (dtype int64): d_out[r]
 * = bytes word*8 .. word*8+7 of row r (compared as int8 when signed_bytes,
 * else as uint8), so ceil(w/8) stable passes, last word first, order the
 * rows as the reference's unique(dim=0) ranks of the rows do (sort.py:31-35). */
int tqpk_string_words(const void* d_src, int64_t n, int32_t width, int32_t word, int32_t signed_bytes,
                      int64_t* d_out, tqpk_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* TQPK_H */
