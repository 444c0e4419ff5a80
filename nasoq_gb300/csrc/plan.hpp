// Plan object behind the C ABI: host symbolic structure, the supernode level
// schedule, the update work lists, and every device buffer of one sparse
// symmetric-indefinite system.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/nasoq_gb300.h"
#include "symbolic.hpp"

namespace nqg {

// Device status bits (plan->d_status).
enum : int {
  ST_ZERO_PIVOT = 1,
  ST_NONFINITE = 2,
  ST_TIMEOUT = 4,
  ST_BOUNDS = 8,
};

// One unit of Schur-update work: the TM x TN block of rows [ri, ri+TM) x
// cols [cj, cj+TN) (positions in descendant d's row list, cols limited to
// <= ub) of L_d D_d L_d^T, subtracted from target supernode s.
struct UpdTile {
  int s, d, ri, cj, ub, q;  // q: the descendant pair
};

// One unit of row-renaming value movement: columns [c0, c0+nc) of the rows
// of descendant pair `pair`; goff >= 0 stages through the global buffer at
// that offset (rows too long for shared memory), else through shared memory.
struct MoveItem {
  int pair, c0, nc, pad;
  int64_t goff;
};

constexpr int RR_STAGE_BYTES = 32 * 1024;       // shared staging of one movement item
constexpr int RR_BIG_STAGE_BYTES = 200 * 1024;  // longest row run staged in shared memory

constexpr int UPD_TM = 64;
constexpr int UPD_TN = 64;
constexpr int UPD_TC_T = 128;       // tensor-core update tiles (FP32 plans)
constexpr int UPD_TC_MIN_WD = 32;   // narrowest descendant whose pairs use them

template <class T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
};

struct Plan {
  // ---- configuration / host structure
  nqg_settings set;
  int n = 0;
  Symbolic sym;
  Csc K;                            // lower CSC, original ordering, values after perturbation
  std::vector<double> Kx_spmv;      // same pattern, perturbed diagonals set to 0 (reference set_diags(0))
  std::vector<int64_t> pert_idx;    // value indices of perturbed diagonals
  double reg32 = 0.0;               // diagonal floor of the FP32 factor
  Csc Uord;                         // upper pattern of the ordered matrix (reach computation)
  std::vector<int> level_of;        // per supernode
  std::vector<std::vector<int>> levels;
  std::vector<int> pair_ptr;        // per supernode s: range of its descendant pairs
  std::vector<int> pair_d, pair_lb, pair_ub;
  std::vector<int64_t> tile_ptr;    // per supernode s: range of its update tiles
  std::vector<UpdTile> tiles;
  std::vector<int64_t> tile_ptr_tc;  // per supernode s: range of its tensor-core update tiles
  std::vector<UpdTile> tiles_tc;
  // FP32: descendant pairs with at least pers_min_flops useful flops run as
  // one persistent tcgen05 launch each on packed operands instead of tiles
  std::vector<int> pers_ptr;        // per supernode s: range in pers_pair
  std::vector<int> pers_pair;       // pair indices
  std::vector<uint8_t> pair_pers;   // per pair: 1 if it is one of them
  // target row positions of every pair's rows lb .. nr-1 (formed per level
  // before its updates, read by the update tiles): offsets per pair
  std::vector<int64_t> pair_moff;
  int64_t map_total = 0;
  int64_t pers_map_ints = 0;        // largest rows + columns of such a pair
  std::vector<int> wide;            // supernodes factored by the blocked kernel
  int64_t ssize = 0;

  // ---- device structure
  cudaStream_t stream = nullptr, own_stream = nullptr;
  int *d_super = nullptr, *d_col2sup = nullptr, *d_ls = nullptr, *d_ls_sym = nullptr;
  int64_t *d_lpi = nullptr, *d_lpx = nullptr;
  int *d_Kp = nullptr, *d_Ki = nullptr;
  double *d_Kx = nullptr;           // factorization copy of K values
  int *d_Rp = nullptr, *d_Rj = nullptr;  // full (both triangles) CSR of K for the SpMV
  double *d_Rx = nullptr;
  int64_t *d_map_lo = nullptr, *d_map_hi = nullptr;  // CSC value index -> CSR positions
  double *d_Kx_spmv = nullptr;      // staging of the refinement values (nqg_set_values)
  int *d_perm = nullptr, *d_iperm = nullptr, *d_locperm = nullptr, *d_perm_tmp = nullptr;
  void *d_L = nullptr;              // factor values (double or float)
  void *d_D = nullptr;              // 2n: diagonal then 2x2 sub-diagonal
  UpdTile *d_tiles = nullptr;
  UpdTile *d_tiles_tc = nullptr;
  int *d_tile_list_tc = nullptr;    // tensor-core tile ids of the current factorization
  size_t tile_list_tc_cap = 0;
  int *d_tile_list = nullptr;       // tile ids for a partial refactor
  size_t tile_list_cap = 0;
  int *d_targets = nullptr;         // supernode ids for per-level kernels
  size_t targets_cap = 0;
  int *d_row_items = nullptr;       // (supernode, row block) pairs of the panel row solves
  size_t row_items_cap = 0;
  int *d_pair_s = nullptr, *d_pair_d = nullptr, *d_pair_lb = nullptr, *d_pair_ub = nullptr;
  // row renaming after pivoting: per-pair row offsets, new positions, moved
  // flags, value-movement items (shared-memory staged, then long rows)
  int *d_locinv = nullptr;          // n: inverse of the in-supernode pivot order
  int64_t *d_pair_roff = nullptr;   // npairs+1: offsets of each pair's rows
  int *d_rr_dest = nullptr;         // new position of every pair row
  uint8_t *d_rr_moved = nullptr;    // npairs: the pair's rows changed order
  MoveItem *d_rr_items = nullptr;
  int64_t rr_items_small = 0, rr_items_big = 0;
  size_t rr_big_smem = 0;           // shared memory of the long-row launch
  void *d_rr_stage = nullptr;       // global staging for rows beyond shared memory
  int rr_words = 0;                 // bitmap words of the widest supernode
  int *d_targets_lv = nullptr;      // narrow supernodes grouped by level (solve kernels)
  std::vector<int> level_off;       // offsets of each level in d_targets_lv
  std::vector<int> lv_targets_host; // host copy of d_targets_lv
  int64_t nnzR = 0;                 // entries of the full CSR used by the SpMV
  // block solves: (supernode, block) items of the large supernodes, per level
  int *d_blk_items = nullptr;       // int pairs: forward items, then backward items
  int *d_flagoff = nullptr;         // per supernode: first of its ready flags
  std::vector<int> blk_fwd_off, blk_bwd_off;  // per level item ranges
  std::vector<double> blk_bytes;    // per level factor entries of the large supernodes
  int solve_small_w = 64;
  std::vector<uint8_t> vis_host;    // host copy of the supernode visibility mask
  double *d_in = nullptr, *d_out = nullptr;  // host-buffer solve staging
  float *d_xf = nullptr;            // FP32 solves: the triangular solves' working vector
  float *d_Z = nullptr;             // FP32 solves: flexible GMRES preconditioned directions
  uint8_t *d_pivoted = nullptr;     // 2*nsuper: [0,ns) BK permuted the supernode in the last factor,
                                    // [ns,2ns) supernode is being factored by the current call
  uint8_t *d_visible = nullptr, *d_hidden = nullptr;
  bool masked = false;
  int *d_status = nullptr;
  // refinement workspace
  double *d_xo = nullptr, *d_bo = nullptr, *d_r = nullptr, *d_V = nullptr, *d_w = nullptr, *d_scal = nullptr;
  int mr_cap = 0;
  // wide supernodes (blocked cooperative BK)
  void *d_wide_W = nullptr;         // panel buffer, max nrow x (nb+2)
  void *d_wide_ctl = nullptr;       // barrier / reduction control block
  unsigned char *d_wide_pack = nullptr;  // FP32: split operand blocks of the tcgen05 updates
  int *d_pers_map = nullptr;              // target positions of a persistent pair's rows and columns
  int *d_pair_map = nullptr;              // target row positions of the pairs' rows (pair_moff)
  int64_t *d_pair_moff = nullptr;
  int *d_map_items = nullptr;             // (pair, first row) items of the per-level map kernel
  size_t map_items_cap = 0;
  unsigned *d_solve_flags = nullptr;  // per 64-column block ready flags of the block solves
  unsigned long long *d_xw = nullptr;  // FP32 block solves: (epoch << 32) | x bits per column
  float *d_tinv = nullptr;             // FP32 block solves: inverses of the diagonal 64 x 64 tiles
  bool tinv_valid = false;             // formed for the current factor
  int solve_flags_cap = 0;
  unsigned solve_epoch = 0;
  int wide_nb = 64;
  int wide_min = 192;               // supernodes wider than this use the blocked kernels
  int bk_small = 64;                // supernodes up to this width: shared-memory BK kernel
  int wide_depth = 8;               // wide supernodes: panels per delayed trailing update (FP32)
  bool panel_rows_serial = false;   // rows below k_bk_global blocks solved inside that kernel
  int num_sms = 0;

  // measurement: launch counter and per-class event timing
  long long nlaunch = 0;
  bool prof = false;
  struct ProfRec {
    int cls;
    cudaEvent_t a, b;
    double flops, bytes;
  };
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  nqg_kernel_stats kstats[NQG_K_CLASSES] = {};
  std::vector<double> pair_flops;   // per descendant pair: useful Schur-update flops
  // Brackets one launch (or one group of launches) of class `cls`.
  cudaEvent_t prof_begin();
  void prof_end(int cls, cudaEvent_t a, double flops, double bytes);
  void prof_collect();
  // Speculative launches: records stay pending while prof_hold is set, and
  // the work of launches that returned without running (queued behind a
  // fast panel that stopped early) is taken back from them.
  bool prof_hold = false;
  size_t prof_mark() const { return prof_pending.size(); }
  void prof_void_from(size_t i) {
    for (size_t k = i; k < prof_pending.size(); ++k) prof_pending[k].flops = prof_pending[k].bytes = 0.0;
  }

  bool factored = false;
  nqg_timings tm{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string last_error;

  size_t val_size() const { return set.precision == NQG_FP32 ? sizeof(float) : sizeof(double); }
};


// numeric.cu
int dev_factor(Plan &P, const std::vector<int> *subset);
// wide.cu
struct WideCtl;
size_t wide_ctl_bytes();
size_t wide_ctl_limit_offset();  // byte offset of the wait limit in the control block
template <class T> int factor_wide(Plan &P, int s, T *L, T *Dg, int nb, T *Wb, WideCtl *ctl, int num_sms);
// Schur update of target s by descendant pair q on the persistent tcgen05
// kernel (FP32 plans).
int update_pair_persistent(Plan &P, int s, int q, float *L, const float *Dg);
// solve_wide.cu
template <class T, class V> int solve_blk_fwd(Plan &P, int level, const T *L, V *x);
template <class T, class V> int solve_blk_bwd(Plan &P, int level, const T *L, V *x);
// solve.cu
int dev_ldlt_solve_ord(Plan &P, double *d_x);
int dev_spmv_ord(Plan &P, const double *d_x_ord, double *d_y_ord);
int dev_spmv_orig(Plan &P, const double *d_x, double *d_y);
int dev_solve(Plan &P, const double *d_rhs, double *d_x);
int dev_refine_only(Plan &P, const double *d_rhs, double *d_x);
int dev_assemble_upload(Plan &P);

#define NQG_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      P.last_error = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
      return NQG_ERR_CUDA;                                                               \
    }                                                                                    \
  } while (0)

}  // namespace nqg
