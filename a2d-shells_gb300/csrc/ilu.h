// Block ILU(k) factorization and level-scheduled triangular solves.
#pragma once
#include <vector>

#include "a2ds_internal.h"

namespace a2ds {

// Rows grouped by dependency level (host copy + device copy of the rows).
struct LevelSchedule {
  int nlevels = 0;
  std::vector<int> ptr;   // nlevels + 1
  std::vector<int> rows;  // rows ordered by level
  DBuf<int> d_rows;
};

// An instantiated CUDA graph of one whole triangular solve, keyed by the
// factor values and the vectors it was captured with.
struct SolveGraph {
  const void *F, *x;
  void *y;
  int nrhs, tv_size;
  cudaGraphExec_t exec;
  long long nlaunch;  // kernels in the graph
};

// Panels: runs of consecutive narrow factor levels whose pivot rows P (at
// most PANEL_MAX_ROWS) are factored together.  Phase 1 runs the panel's
// levels restricted to target rows in P; phase 2 updates every other target
// row with all of P's pivots in one pass (one task per row).
struct PanelSchedule {
  std::vector<int> level_panel;  // per factor level: its panel, -1 if none
  std::vector<int> l0, l1;       // level range [l0, l1) of each panel
  std::vector<int> np;           // pivot rows of each panel
  std::vector<int> task_np;      // per level: leading tasks with targets in P
  std::vector<int> prow;         // PANEL_MAX_ROWS per panel: P in level order (-1 pad)
  // union of the U columns of P outside P, sorted, per panel
  std::vector<int> uc_ptr, uc;
  // per panel np x nuc: U position of pivot k at column uc[u] (-1: none)
  std::vector<int> tab_off, tab;
  // PANEL_MAX_ROWS^2 per panel: U position of pivot k at column prow[k2]
  std::vector<int> tp;
  // phase-2 tasks: per panel a range of target rows; PANEL_MAX_ROWS L
  // positions per task (L block of the row in column prow[k], -1: none)
  std::vector<int> task_ptr, task_row, task_jpk;
  std::vector<int> task_maxlen;  // per panel: longest target row of its phase-2 tasks
};

// Chunked triangular solves.  Rows are cut into chunks of consecutive rows:
// a chunk ends before row i when row i has no L block in column i - 1, or
// when it reaches CHUNK_MAX rows.  Within a chunk every row may depend on
// the earlier ones, so its diagonal block is solved as one dense operator
// (the inverse of its unit-lower part and of its D + U part, built after
// the numeric factorization); the chunk's other factor blocks point to
// earlier chunks (lower) or later ones (upper).  Chunks are scheduled by
// dependency levels over those external columns: one launch pulls the
// external sums of every row of the level (each row's external blocks cut
// into segments of at most SOLVE_SEG blocks, one warp per segment, the
// segments of one row adding atomically), one applies the chunk inverses.
// On the AMD-ordered cylinders this gives 16 levels at 256x512 and 43 at
// 512x1024 (CHUNK_MAX 128), against 1,893 and 3,810 row levels.
struct ChunkLevels {
  int nlevels = 0;
  std::vector<int> row_ptr, rows;   // rows of each level
  // pull segments of each level: row, block range [kb, ke), flags (bit 0:
  // the row has more than one segment, so they add atomically)
  std::vector<int> seg_ptr, seg_row, seg_kb, seg_ke, seg_flag;
  // upper levels: one-row chunks whose pull is segmented, finished by the
  // apply launch (y_i = D_i^{-1} t_i)
  std::vector<int> fin_ptr, fin_rows;
  std::vector<int> ch_ptr, chunks;  // chunks of >= 2 rows of each level, those of more
                                    // than APPLY_WARP_ROWS rows first
  std::vector<int> nbig;            // per level: chunks of more than APPLY_WARP_ROWS rows
  std::vector<int> max_rows;        // per level: rows of its largest chunk
};
struct ChunkPlan {
  std::vector<int> c0;          // chunk starts (nchunks + 1 entries, last = n)
  std::vector<long long> off;   // per chunk: offset of its L inverse ((6 ns)^2 values,
                                // row-major), the U inverse follows; -1 for one row
  long long inv_size = 0;       // values of all inverses
  long long scr_size = 0;       // values of all gathered diagonal blocks
  int max_rows = 0;             // largest chunk
  std::vector<int> row_lend;    // per row: end of its lower pull (first column >= its chunk)
  std::vector<int> row_ustart;  // per row: start of its upper pull (first column past its chunk)
  std::vector<int> row_single;  // per row: 1 if its chunk is the row alone
  ChunkLevels lo, up;           // up: level 0 solved first (top of the ordering)
  std::vector<int> small, big;  // multi-row chunks of at most / more than 10 rows
};

// A factorization handle (the TACSSchurPc role on one GPU).
struct Factor {
  int n = 0, lev_fill = 0, precision = 64;
  bool df_compute = false;  // FP32 factor computed in double-float (factor_df_to_f32)
  std::vector<int> frowp, fcols, fdiag;
  DBuf<int> d_frowp, d_fcols, d_fdiag, d_status;
  DBuf<double> F64;
  DBuf<float> F32;
  LevelSchedule flv;           // dependency levels of all rows (factorization)
  // right-looking update tasks, grouped by level; within a level the tasks
  // of long target rows (> FACTOR_WARP_COLS blocks) come first
  std::vector<int> task_level_ptr, task_nlong, task_row, task_ptr, task_jp;
  std::vector<int> task_long_cols;  // per level: longest target row of its long tasks
  std::vector<int> task_group;  // block updates in flight per short task, per level (1, 2, 5)
  // panels of narrow levels (blocked trailing updates, see build_update_tasks)
  PanelSchedule pn;
  DBuf<int> d_pn_prow, d_pn_uc, d_pn_tab, d_pn_tp, d_pn_task_row, d_pn_task_jpk;
  DBuf<int> d_task_row, d_task_ptr, d_task_jp;
  // Chunked triangular solves (see ChunkPlan); host plan, device copies and
  // the inverses of the chunks' diagonal blocks (rebuilt after every
  // numeric factorization)
  ChunkPlan cp;
  DBuf<int> d_ck_c0, d_row_lend, d_row_ustart, d_row_single;
  DBuf<long long> d_ck_off;
  DBuf<int> d_lo_chunks, d_up_chunks, d_ck_small, d_ck_big;
  DBuf<int> d_lo_seg_row, d_lo_seg_kb, d_lo_seg_ke, d_lo_seg_flag;
  DBuf<int> d_up_seg_row, d_up_seg_kb, d_up_seg_ke, d_up_seg_flag, d_up_fin;
  DBuf<double> cinv64, cscr64;  // FP64 inverses (all precisions) and gathered blocks
  DBuf<float> cinv32;           // FP32 copy of the inverses for FP32 factors
  DBuf<unsigned char> tvec;     // solve scratch: the pulled sums of chunk rows
  // algorithmic FP operations of one numeric factorization: 432 per L block
  // (L_ij = A_ij D_j^{-1}), 432 per block update, 432 per diagonal inverse
  double flop_count = 0.0;
  std::vector<SolveGraph> graphs;  // solve_graph cache (at most 8)
  Factor() = default;
  ~Factor();
  long long nnzb() const { return frowp.empty() ? 0 : frowp.back(); }
  double flops() const { return flop_count; }
};

void build_levels(int n, const std::vector<int> &frowp, const std::vector<int> &fcols,
                  const std::vector<int> &fdiag, bool upper, LevelSchedule &L,
                  std::vector<int> *level_of = nullptr);
void build_update_tasks(Factor &f, const std::vector<int> &lev);
// The chunked solve plan of f's pattern (ChunkPlan).
void build_solve_schedule(Factor &f);
int upload_schedules(Factor &f, cudaStream_t s);
// Allocate the chunk-inverse buffers of f for its precision.
int chunk_alloc(Factor &f);
// Gather every chunk's diagonal block out of the factored values F and
// invert its unit-lower and D + U parts (after the numeric factorization).
int chunk_build(Factor &f, const void *F, cudaStream_t s, long long *launches);

// Update kernels: tasks on target rows with at most FACTOR_WARP_COLS
// blocks, or with fewer than FACTOR_LONG_WORK block updates, go to a group
// of 6, 12 or 30 lanes; the rest to one CTA each (column indices staged in
// shared memory up to FACTOR_CTA_COLS).
constexpr int FACTOR_WARP_COLS = 512;
// block updates below which a task on a long target row still goes to the
// warp-group kernel (a 384-thread CTA applies 64 block updates at a time)
constexpr long long FACTOR_LONG_WORK = 256;
constexpr int FACTOR_CTA_COLS = 10240;
// at most this many CTAs share one single-pivot long update task
constexpr int FACTOR_MAX_SPLIT = 8;
// Panels of the factorization: runs of levels with at most PANEL_LEVEL_ROWS
// rows each, PANEL_MAX_ROWS rows in total.
constexpr int PANEL_LEVEL_ROWS = 32;
constexpr int PANEL_MAX_ROWS = 64;
// upper bound on the panel tables' entries (a bound on host and device
// memory, 1 GB of int32; runs of levels past it are factored level by level)
constexpr long long PANEL_TABLE_MAX = 1LL << 28;
// union U columns of a panel staged in shared memory by its phase-2 kernel
constexpr int PANEL_UC_SMEM = 8192;

// Largest chunk of the solves (block rows), and the factor blocks of one
// pull segment (one warp: five groups of six lanes, four blocks per step).
constexpr int CHUNK_MAX = 128;
constexpr int SOLVE_SEG = 40;
// chunks of at most this many rows are applied one warp per chunk
constexpr int APPLY_WARP_ROWS = 16;

// F (f.precision: 64 double, 48 double-float, 32 float values; 8 bytes per
// value for 64 and 48) <- pattern-embedded copy of A (+ alpha2 * A2 when
// A2 != NULL).
int factor_scatter(const Factor &f, int n, const int *rowp, const int *cols, const double *A,
                   const double *A2, double alpha2, void *F, cudaStream_t s);

// In-place numeric factorization of F.  *status receives max(row+1) of any
// singular diagonal block (0 = none).  A double-float factor is converted to
// FP64 in place at the end.
int factor_levels(const Factor &f, void *F, int *status, cudaStream_t s, long long *launches);
// An FP32 factor (f.F32) computed in double-float arithmetic: the scatter
// and the level-scheduled factorization run on df64 values in work (8 bytes
// per value, nnzb_f x 36), then every value is rounded to FP32 once, so the
// FP32 factor carries one rounding instead of the FP32 factorization's
// accumulated errors.
int factor_df_to_f32(const Factor &f, int n, const int *rowp, const int *cols, const double *A,
                     const double *A2, double alpha2, void *work, float *F32, int *status,
                     cudaStream_t s, long long *launches);

// y = (LU)^{-1} x for nrhs in {1, 2, 4, 8, 16} right-hand sides, layout
// (row, dof, rhs); y may alias x.  solve_levels launches the level kernels
// on s; solve_graph does the same through a CUDA graph captured on the
// first call with these (F, x, y, nrhs) and replayed afterwards (s must not
// be capturing already).
template <typename T, typename TV>
int solve_levels(Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                 long long *launches);
template <typename T, typename TV>
int solve_graph(Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                long long *launches);

struct Mesh;
int factor_setup(Mesh &m, int lev_fill, int precision, Factor &f);
// Factor A (+ alpha2 * A2) -- both in the mesh pattern -- into f.
int factor_numeric(Mesh &m, Factor &f, const double *A, const double *A2, double alpha2);
int factor_check(Mesh &m, Factor &f);  // reads the singular-pivot status

}  // namespace a2ds
