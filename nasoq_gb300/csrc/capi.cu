// extern "C" entry points of include/nasoq_gb300.h: plan construction (host
// symbolic analysis, level schedule, update work lists, device uploads) and
// the factor / solve calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "plan.hpp"

using namespace nqg;

struct nqg_symbolic {
  Symbolic sym;
};
struct nqg_plan {
  Plan P;
};

extern "C" void nqg_default_settings(nqg_settings *s) {
  if (!s) return;
  s->precision = NQG_FP64;
  s->req_ref_iter = 2;
  s->max_inner_iter = 2;
  s->tol_abs = 1e-15;
  s->tol_rel = 1e-15;
  s->reg_diag = 1e-8;
  s->regularization = 1;
  s->n_relax[0] = 4;
  s->n_relax[1] = 16;
  s->n_relax[2] = 48;
  s->z_relax[0] = 0.8;
  s->z_relax[1] = 0.1;
  s->z_relax[2] = 0.05;
  s->reg_diag_fp32 = 0.0;
  s->solve_precision = NQG_FP64;
  s->perturb_plus_cols = -1;
}

extern "C" const char *nqg_status_str(int st) {
  switch (st) {
    case NQG_OK: return "ok";
    case NQG_WARN_ZERO_PIVOT: return "factorization met an exactly singular pivot block";
    case NQG_WARN_NONFINITE: return "factorization produced a non-finite value";
    case NQG_ERR_ARG: return "invalid argument";
    case NQG_ERR_CUDA: return "CUDA error";
    case NQG_ERR_SYMBOLIC: return "symbolic analysis failed";
    case NQG_ERR_STATE: return "call out of order";
    case NQG_ERR_TIMEOUT: return "device wait timed out";
    case NQG_ERR_SIZE: return "problem exceeds a fixed capacity";
    default: return "unknown status";
  }
}

static bool check_lower_csc(int n, const int *Ap, const int *Ai) {
  if (n < 0 || (n > 0 && (!Ap || !Ai))) return false;
  if (n == 0) return true;
  if (Ap[0] != 0) return false;
  for (int j = 0; j < n; ++j) {
    // every column stores its diagonal first (reference find_perturbation and
    // set_diags address A->x[A->p[j]] as the diagonal)
    if (Ap[j + 1] <= Ap[j] || Ai[Ap[j]] != j) return false;
    for (int q = Ap[j]; q < Ap[j + 1]; ++q) {
      if (Ai[q] < j || Ai[q] >= n) return false;
      if (q > Ap[j] && Ai[q] <= Ai[q - 1]) return false;
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// symbolic only
extern "C" int nqg_symbolic_create(int n, const int *Ap, const int *Ai, const int *extra_cols, const int n_relax[3],
                                   const double z_relax[3], nqg_symbolic **out) {
  if (!out || !check_lower_csc(n, Ap, Ai)) return NQG_ERR_ARG;
  *out = nullptr;
  Csc A;
  A.n = n;
  A.p.assign(Ap, Ap + n + 1);
  A.i.assign(Ai, Ai + Ap[n]);
  int nr[3] = {4, 16, 48};
  double zr[3] = {0.8, 0.1, 0.05};
  if (n_relax) std::copy(n_relax, n_relax + 3, nr);
  if (z_relax) std::copy(z_relax, z_relax + 3, zr);
  auto *h = new (std::nothrow) nqg_symbolic;
  if (!h) return NQG_ERR_SIZE;
  std::string err = analyze(A, extra_cols, nr, zr, h->sym);
  if (!err.empty()) {
    delete h;
    return NQG_ERR_SYMBOLIC;
  }
  *out = h;
  return NQG_OK;
}

static void fill_info(const Symbolic &S, nqg_symbolic_info *info) {
  info->n = S.n;
  info->nsuper = S.nsuper;
  info->max_sup_wid = S.max_sup_wid;
  info->max_col = S.max_col;
  info->ssize = S.nsuper > 0 ? S.lpi[S.nsuper] : 0;
  info->xsize = S.xsize;
  info->metis_seconds = S.metis_seconds;
  info->total_seconds = S.total_seconds;
}

extern "C" int nqg_symbolic_get_info(const nqg_symbolic *h, nqg_symbolic_info *info) {
  if (!h || !info) return NQG_ERR_ARG;
  fill_info(h->sym, info);
  return NQG_OK;
}

static void export_sym(const Symbolic &S, int *perm, int *iperm, int *parent, int *colcount, int *super, int *sparent,
                       int *col2sup, int64_t *lpi, int *ls, int64_t *colp, int *extra) {
  const int n = S.n, ns = S.nsuper;
  if (perm) std::copy(S.perm.begin(), S.perm.end(), perm);
  if (iperm) std::copy(S.iperm.begin(), S.iperm.end(), iperm);
  if (parent) std::copy(S.parent.begin(), S.parent.end(), parent);
  if (colcount) std::copy(S.colcount.begin(), S.colcount.end(), colcount);
  if (super) std::copy(S.super.begin(), S.super.begin() + ns + 1, super);
  if (sparent) std::copy(S.sparent.begin(), S.sparent.end(), sparent);
  if (col2sup) std::copy(S.col2sup.begin(), S.col2sup.end(), col2sup);
  if (lpi) std::copy(S.lpi.begin(), S.lpi.end(), lpi);
  if (ls && ns > 0) std::copy(S.ls.begin(), S.ls.begin() + S.lpi[ns], ls);
  if (colp) std::copy(S.colp.begin(), S.colp.begin() + n + 1, colp);
  if (extra) std::copy(S.extra_cols.begin(), S.extra_cols.end(), extra);
}

extern "C" int nqg_symbolic_export(const nqg_symbolic *h, int *perm, int *iperm, int *parent, int *colcount,
                                   int *super, int *sparent, int *col2sup, int64_t *lpi, int *ls, int64_t *colp,
                                   int *extra_cols) {
  if (!h) return NQG_ERR_ARG;
  export_sym(h->sym, perm, iperm, parent, colcount, super, sparent, col2sup, lpi, ls, colp, extra_cols);
  return NQG_OK;
}

extern "C" void nqg_symbolic_destroy(nqg_symbolic *h) { delete h; }

// ---------------------------------------------------------------------------
// plan construction helpers

// Supernode levels (leaves 0), descendant pairs from the elimination-tree
// reach of every supernode, and the 64x64 update tiles of each pair.
static void build_schedule(Plan &P) {
  Symbolic &S = P.sym;
  const int ns = S.nsuper;
  P.level_of.assign(ns, 0);
  int maxlev = 0;
  for (int s = 0; s < ns; ++s) {
    int p = S.sparent[s];
    if (p >= 0) P.level_of[p] = std::max(P.level_of[p], P.level_of[s] + 1);
    maxlev = std::max(maxlev, P.level_of[s]);
  }
  P.levels.assign(ns > 0 ? maxlev + 1 : 0, {});
  for (int s = 0; s < ns; ++s) P.levels[P.level_of[s]].push_back(s);
  // pairs
  std::vector<int> mark(ns, 0), stack, lst;
  P.pair_ptr.assign(ns + 1, 0);
  P.pair_d.clear();
  P.pair_lb.clear();
  P.pair_ub.clear();
  P.pair_flops.clear();
  P.pair_pers.clear();
  P.pair_moff.clear();
  P.map_total = 0;
  P.tile_ptr.assign(ns + 1, 0);
  P.tiles.clear();
  P.tile_ptr_tc.assign(ns + 1, 0);
  P.tiles_tc.clear();
  P.pers_ptr.assign(ns + 1, 0);
  P.pers_pair.clear();
  P.pers_map_ints = 0;
  // FP32 plans: pairs whose descendant has at least UPD_TC_MIN_WD columns
  // (NASOQ_GB300_UPDATE_TC_MIN overrides) take 128 x 128 tensor-core tiles;
  // NASOQ_GB300_UPDATE=simt keeps them all on the CUDA-core kernel
  const char *ue = std::getenv("NASOQ_GB300_UPDATE");
  const bool tc = P.set.precision == NQG_FP32 && !(ue && std::string(ue) == "simt");
  int tc_min_wd = UPD_TC_MIN_WD;
  if (const char *e = std::getenv("NASOQ_GB300_UPDATE_TC_MIN")) tc_min_wd = std::max(1, std::atoi(e));
  // pairs of at least this many useful flops go to the persistent kernel
  // (NASOQ_GB300_UPDATE_PERSIST_MIN; a negative value keeps every pair on tiles)
  double pers_min = 1e10;
  if (const char *e = std::getenv("NASOQ_GB300_UPDATE_PERSIST_MIN")) pers_min = std::atof(e);
  for (int s = 0; s < ns; ++s) {
    ereach_sn(S, P.Uord, s, S.sparent, mark, stack, lst);
    const int c1 = S.super[s], c2 = S.super[s + 1];
    for (int d : lst) {
      const int *rows = S.ls.data() + S.lpi[d];
      const int nr = (int)(S.lpi[d + 1] - S.lpi[d]);
      int lb = (int)(std::lower_bound(rows, rows + nr, c1) - rows);
      int ub = (int)(std::lower_bound(rows, rows + nr, c2) - rows) - 1;
      if (lb >= nr || ub < lb) continue;  // no overlap (cannot happen for a true reach)
      P.pair_d.push_back(d);
      P.pair_lb.push_back(lb);
      P.pair_ub.push_back(ub);
      {
        // useful multiply-adds: lower trapezoid of the (nr-lb) x (ub-lb+1) block, depth = width of d
        const double m = nr - lb, nc = ub - lb + 1, wd = S.super[d + 1] - S.super[d];
        P.pair_flops.push_back(2.0 * wd * (nc * m - nc * (nc - 1) / 2.0));
        P.pair_pers.push_back(0);
        P.pair_moff.push_back(P.map_total);
        P.map_total += nr - lb;
      }
      if (tc && S.super[d + 1] - S.super[d] >= tc_min_wd && pers_min >= 0 && P.pair_flops.back() >= pers_min) {
        P.pers_pair.push_back((int)P.pair_d.size() - 1);
        P.pair_pers.back() = 1;
        P.pers_map_ints = std::max<int64_t>(P.pers_map_ints, (int64_t)(nr - lb) + (ub - lb + 1));
      } else if (tc && S.super[d + 1] - S.super[d] >= tc_min_wd) {
        for (int ri = lb; ri < nr; ri += UPD_TC_T)
          for (int cj = lb; cj <= ub; cj += UPD_TC_T)
            if (ri + UPD_TC_T - 1 >= cj) P.tiles_tc.push_back(UpdTile{s, d, ri, cj, ub, (int)P.pair_d.size() - 1});
      } else {
        for (int ri = lb; ri < nr; ri += UPD_TM)
          for (int cj = lb; cj <= ub; cj += UPD_TN)
            if (ri + UPD_TM - 1 >= cj) P.tiles.push_back(UpdTile{s, d, ri, cj, ub, (int)P.pair_d.size() - 1});
      }
    }
    P.pair_ptr[s + 1] = (int)P.pair_d.size();
    P.tile_ptr[s + 1] = (int64_t)P.tiles.size();
    P.tile_ptr_tc[s + 1] = (int64_t)P.tiles_tc.size();
    P.pers_ptr[s + 1] = (int)P.pers_pair.size();
  }
}

template <class T> static int dev_alloc_copy(Plan &P, T **dst, const T *src, size_t count) {
  NQG_CUDA(cudaMalloc(dst, std::max<size_t>(count, 1) * sizeof(T)));
  if (count) NQG_CUDA(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return NQG_OK;
}

// Full CSR (both triangles) of K with the refinement values; map_lo/map_hi
// give, for every lower-CSC entry, its positions in the CSR (hi = -1 on the
// diagonal).
static void build_full_csr(const Csc &K, const std::vector<double> &xv, std::vector<int> &Rp, std::vector<int> &Rj,
                           std::vector<double> &Rx, std::vector<int64_t> &mlo, std::vector<int64_t> &mhi) {
  const int n = K.n;
  Rp.assign(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
      int i = K.i[q];
      Rp[i + 1]++;
      if (i != j) Rp[j + 1]++;
    }
  for (int i = 0; i < n; ++i) Rp[i + 1] += Rp[i];
  Rj.resize(Rp[n]);
  Rx.resize(Rp[n]);
  mlo.assign(K.nnz(), -1);
  mhi.assign(K.nnz(), -1);
  std::vector<int> pos(Rp.begin(), Rp.end() - 1);
  // entries of row i: columns j <= i come from column j (lower), in increasing j;
  // columns j > i come from column i itself.  Visit columns in order.
  for (int j = 0; j < n; ++j)
    for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
      int i = K.i[q];
      int t = pos[i]++;
      Rj[t] = j;
      Rx[t] = xv[q];
      mlo[q] = t;
    }
  for (int j = 0; j < n; ++j)
    for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
      int i = K.i[q];
      if (i == j) continue;
      int t = pos[j]++;
      Rj[t] = i;
      Rx[t] = xv[q];
      mhi[q] = t;
    }
}

static int upload_plan(Plan &P) {
  Symbolic &S = P.sym;
  const int n = P.n, ns = S.nsuper;
  if (!P.own_stream) NQG_CUDA(cudaStreamCreateWithFlags(&P.own_stream, cudaStreamNonBlocking));
  P.stream = P.own_stream;
  NQG_CUDA(cudaEventCreate(&P.ev0));
  NQG_CUDA(cudaEventCreate(&P.ev1));
  int rc;
  if ((rc = dev_alloc_copy(P, &P.d_super, S.super.data(), S.super.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_col2sup, S.col2sup.data(), S.col2sup.size()))) return rc;
  P.ssize = ns > 0 ? S.lpi[ns] : 0;
  if ((rc = dev_alloc_copy(P, &P.d_ls, S.ls.data(), (size_t)P.ssize))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_ls_sym, S.ls.data(), (size_t)P.ssize))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_lpi, S.lpi.data(), S.lpi.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_lpx, S.lpx.data(), S.lpx.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_Kp, P.K.p.data(), P.K.p.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_Ki, P.K.i.data(), P.K.i.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_Kx, P.K.x.data(), P.K.x.size()))) return rc;
  std::vector<int> Rp, Rj;
  std::vector<double> Rx;
  std::vector<int64_t> mlo, mhi;
  build_full_csr(P.K, P.Kx_spmv, Rp, Rj, Rx, mlo, mhi);
  if ((rc = dev_alloc_copy(P, &P.d_Rp, Rp.data(), Rp.size()))) return rc;
  P.nnzR = Rp.back();
  if ((rc = dev_alloc_copy(P, &P.d_Rj, Rj.data(), Rj.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_Rx, Rx.data(), Rx.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_map_lo, mlo.data(), mlo.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_map_hi, mhi.data(), mhi.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_perm, S.perm.data(), S.perm.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_iperm, S.iperm.data(), S.iperm.size()))) return rc;
  NQG_CUDA(cudaMalloc(&P.d_locperm, std::max(n, 1) * sizeof(int)));
  NQG_CUDA(cudaMalloc(&P.d_perm_tmp, std::max(n, 1) * sizeof(int)));
  NQG_CUDA(cudaMalloc(&P.d_L, (size_t)S.xsize * P.val_size()));
  NQG_CUDA(cudaMalloc(&P.d_D, (size_t)std::max(2 * n, 2) * P.val_size()));
  NQG_CUDA(cudaMemset(P.d_L, 0, (size_t)S.xsize * P.val_size()));
  NQG_CUDA(cudaMemset(P.d_D, 0, (size_t)std::max(2 * n, 2) * P.val_size()));
  if ((rc = dev_alloc_copy(P, &P.d_tiles, P.tiles.data(), P.tiles.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_tiles_tc, P.tiles_tc.data(), P.tiles_tc.size()))) return rc;
  std::vector<int> ps(P.pair_d.size());
  for (int s = 0; s < ns; ++s)
    for (int q = P.pair_ptr[s]; q < P.pair_ptr[s + 1]; ++q) ps[q] = s;
  if ((rc = dev_alloc_copy(P, &P.d_pair_s, ps.data(), ps.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_pair_d, P.pair_d.data(), P.pair_d.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_pair_lb, P.pair_lb.data(), P.pair_lb.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_pair_moff, P.pair_moff.data(), P.pair_moff.size()))) return rc;
  NQG_CUDA(cudaMalloc(&P.d_pair_map, (size_t)std::max<int64_t>(P.map_total, 1) * sizeof(int)));
  if ((rc = dev_alloc_copy(P, &P.d_pair_ub, P.pair_ub.data(), P.pair_ub.size()))) return rc;
  {
    // row renaming work: rows of every pair, and value-movement items sized so
    // one item's rows x columns fit the shared-memory staging buffer
    const int64_t np = (int64_t)P.pair_d.size();
    std::vector<int64_t> roff(np + 1, 0);
    for (int64_t q = 0; q < np; ++q) roff[q + 1] = roff[q] + std::max(0, P.pair_ub[q] - P.pair_lb[q] + 1);
    const int64_t cap = RR_STAGE_BYTES / (int64_t)P.val_size();
    const int64_t big_cap = RR_BIG_STAGE_BYTES / (int64_t)P.val_size();
    std::vector<MoveItem> small, big;
    int64_t goff = 0, big_len = 0;
    for (int64_t q = 0; q < np; ++q) {
      const int len = P.pair_ub[q] - P.pair_lb[q] + 1;
      const int d = P.pair_d[q];
      const int wd = S.super[d + 1] - S.super[d];
      if (len <= 0 || wd <= 0) continue;
      if (len <= cap) {
        const int cc = (int)std::max<int64_t>(1, cap / len);
        for (int c = 0; c < wd; c += cc) small.push_back({(int)q, c, std::min(cc, wd - c), 0, -1});
      } else {
        for (int c = 0; c < wd; ++c) {
          int64_t g = -1;
          if (len > big_cap) {
            g = goff;
            goff += len;
          } else {
            big_len = std::max<int64_t>(big_len, len);
          }
          big.push_back({(int)q, c, 1, 0, g});
        }
      }
    }
    P.rr_items_small = (int64_t)small.size();
    P.rr_items_big = (int64_t)big.size();
    P.rr_big_smem = (size_t)big_len * P.val_size();
    small.insert(small.end(), big.begin(), big.end());
    if ((rc = dev_alloc_copy(P, &P.d_pair_roff, roff.data(), roff.size()))) return rc;
    if ((rc = dev_alloc_copy(P, &P.d_rr_items, small.data(), small.size()))) return rc;
    NQG_CUDA(cudaMalloc(&P.d_rr_dest, (size_t)std::max<int64_t>(roff[np], 1) * sizeof(int)));
    NQG_CUDA(cudaMalloc(&P.d_rr_moved, (size_t)std::max<int64_t>(np, 1)));
    NQG_CUDA(cudaMalloc(&P.d_locinv, std::max(n, 1) * sizeof(int)));
    if (goff > 0) NQG_CUDA(cudaMalloc(&P.d_rr_stage, (size_t)goff * P.val_size()));
    P.rr_words = (std::max(S.max_sup_wid, 1) + 31) / 32;
  }
  // tuning overrides: width above which the blocked multi-CTA kernels take
  // a supernode, and their panel width
  if (const char *e = std::getenv("NASOQ_GB300_WIDE_MIN")) P.wide_min = std::max(1, std::atoi(e));
  if (const char *e = std::getenv("NASOQ_GB300_WIDE_NB")) P.wide_nb = std::min(64, std::max(4, std::atoi(e)));
  // supernodes of at most this width take the shared-memory BK kernel (<= 64)
  if (const char *e = std::getenv("NASOQ_GB300_BK_SMALL")) P.bk_small = std::min(64, std::max(1, std::atoi(e)));
  // panels per delayed trailing update of the FP32 wide supernodes (1..8)
  if (const char *e = std::getenv("NASOQ_GB300_WIDE_DEPTH")) P.wide_depth = std::min(8, std::max(1, std::atoi(e)));
  // =serial: the rows below the k_bk_global blocks are solved in that kernel
  if (const char *e = std::getenv("NASOQ_GB300_PANEL_ROWS")) P.panel_rows_serial = std::string(e) == "serial";
  // solve work split per level: small supernodes take one CTA each in the
  // level kernels; the others are cut into 64-row blocks for the
  // flag-driven block kernels (forward items: diagonal block rows, then row
  // blocks below; backward items: diagonal column blocks)
  int small_w = 64, small_rows = 256;
  if (const char *e = std::getenv("NASOQ_GB300_SOLVE_SMALL")) std::sscanf(e, "%d,%d", &small_w, &small_rows);
  std::vector<int> lvflat, flagoff(std::max(ns, 1), 0), fwd_items, bwd_items;
  P.level_off.assign(P.levels.size() + 1, 0);
  P.blk_fwd_off.assign(P.levels.size() + 1, 0);
  P.blk_bwd_off.assign(P.levels.size() + 1, 0);
  P.blk_bytes.assign(P.levels.size(), 0.0);
  int nflags = 0;
  for (size_t l = 0; l < P.levels.size(); ++l) {
    for (int s : P.levels[l]) {
      const int w = S.super[s + 1] - S.super[s];
      const int nrow = (int)(S.lpi[s + 1] - S.lpi[s]);
      if (w <= small_w && nrow <= small_rows) {
        lvflat.push_back(s);
        continue;
      }
      const int nbd = (w + 63) / 64, nbb = (nrow - w + 63) / 64;
      flagoff[s] = nflags;
      nflags += nbd;
      for (int q = 0; q < nbd + nbb; ++q) {
        fwd_items.push_back(s);
        fwd_items.push_back(q);
      }
      for (int q = 0; q < nbd; ++q) {
        bwd_items.push_back(s);
        bwd_items.push_back(q);
      }
      P.blk_bytes[l] += (double)nrow * w;
    }
    P.level_off[l + 1] = (int)lvflat.size();
    P.blk_fwd_off[l + 1] = (int)fwd_items.size() / 2;
    P.blk_bwd_off[l + 1] = (int)bwd_items.size() / 2;
  }
  const int nfwd = (int)fwd_items.size() / 2;
  for (auto &o : P.blk_bwd_off) o += nfwd;
  fwd_items.insert(fwd_items.end(), bwd_items.begin(), bwd_items.end());
  if ((rc = dev_alloc_copy(P, &P.d_blk_items, fwd_items.data(), fwd_items.size()))) return rc;
  if ((rc = dev_alloc_copy(P, &P.d_flagoff, flagoff.data(), flagoff.size()))) return rc;
  P.solve_flags_cap = std::max(nflags, 1);
  NQG_CUDA(cudaMalloc(&P.d_solve_flags, (size_t)P.solve_flags_cap * sizeof(unsigned)));
  NQG_CUDA(cudaMemset(P.d_solve_flags, 0, (size_t)P.solve_flags_cap * sizeof(unsigned)));
  NQG_CUDA(cudaMalloc(&P.d_xw, (size_t)std::max(n, 1) * sizeof(unsigned long long)));
  NQG_CUDA(cudaMemset(P.d_xw, 0, (size_t)std::max(n, 1) * sizeof(unsigned long long)));
  // FP32 factor with FP32 block solves: per diagonal tile (one per ready
  // flag) its inverse and the two last-link products, 64 x 65 floats each
  if (P.set.precision == NQG_FP32 && P.set.solve_precision == NQG_FP32)
    NQG_CUDA(cudaMalloc(&P.d_tinv, (size_t)std::max(nflags, 1) * 3 * 64 * 65 * sizeof(float)));
  P.solve_small_w = small_w;
  if ((rc = dev_alloc_copy(P, &P.d_targets_lv, lvflat.data(), lvflat.size()))) return rc;
  P.lv_targets_host = lvflat;
  P.vis_host.assign(ns, 1);
  NQG_CUDA(cudaMalloc(&P.d_pivoted, std::max(2 * ns, 2)));
  NQG_CUDA(cudaMemset(P.d_pivoted, 0, std::max(2 * ns, 2)));
  NQG_CUDA(cudaMalloc(&P.d_visible, std::max(ns, 1)));
  NQG_CUDA(cudaMalloc(&P.d_hidden, std::max(n, 1)));
  NQG_CUDA(cudaMalloc(&P.d_status, sizeof(int)));
  NQG_CUDA(cudaMemset(P.d_status, 0, sizeof(int)));
  P.mr_cap = std::max(P.set.max_inner_iter, 8);
  const size_t nn = std::max(n, 1);
  NQG_CUDA(cudaMalloc(&P.d_xo, nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_bo, nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_r, nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_w, nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_in, nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_out, nn * sizeof(double)));
  if (P.set.precision == NQG_FP32 && P.set.solve_precision == NQG_FP32) {
    NQG_CUDA(cudaMalloc(&P.d_xf, nn * sizeof(float)));
    NQG_CUDA(cudaMalloc(&P.d_Z, (size_t)P.mr_cap * nn * sizeof(float)));
  }
  NQG_CUDA(cudaMalloc(&P.d_V, (size_t)(P.mr_cap + 1) * nn * sizeof(double)));
  NQG_CUDA(cudaMalloc(&P.d_scal, (64 + 512) * sizeof(double)));
  {
    int dev = 0;
    NQG_CUDA(cudaGetDevice(&dev));
    NQG_CUDA(cudaDeviceGetAttribute(&P.num_sms, cudaDevAttrMultiProcessorCount, dev));
    int64_t wide_rows = 0;
    for (int s = 0; s < ns; ++s)
      if (S.super[s + 1] - S.super[s] > P.wide_min) wide_rows = std::max<int64_t>(wide_rows, S.lpi[s + 1] - S.lpi[s]);
    // W of up to wide_depth + 1 pending panels (each at most nb + 1 columns)
    // plus the two working columns of the panel kernel
    if (wide_rows > 0)
      NQG_CUDA(cudaMalloc(&P.d_wide_W,
                          (size_t)wide_rows * ((P.wide_depth + 1) * (P.wide_nb + 1) + 2) * P.val_size()));
    // FP32: packed split operands of the persistent tcgen05 updates, blocks
    // of 128 rows x one chunk of K (hi + lo halves of 16 KB each; counted
    // here in 32-entry TF32 chunks, at least as many as 64-entry BF16 ones).
    // Trailing updates of a wide supernode: row blocks of L then of W, each
    // wide_depth panels of chunks; a persistent descendant pair: row blocks
    // of L D then of L, the descendant's width in chunks.  One buffer serves
    // both (they never run at the same time).
    if (P.set.precision == NQG_FP32) {
      int64_t chunks = 0;
      if (wide_rows > 0) {
        int64_t blocks = 0;
        for (int s = 0; s < ns; ++s)
          if (S.super[s + 1] - S.super[s] > P.wide_min)
            blocks = std::max<int64_t>(blocks, (S.lpi[s + 1] - S.lpi[s] + 127) / 128 +
                                                   (S.super[s + 1] - S.super[s] + 127) / 128);
        chunks = blocks * (int64_t)(std::max(P.wide_depth, 1) + 1) * ((P.wide_nb + 1 + 31) / 32);
      }
      for (int q : P.pers_pair) {
        const int d = P.pair_d[q];
        const int64_t m = (S.lpi[d + 1] - S.lpi[d]) - P.pair_lb[q], nc = P.pair_ub[q] - P.pair_lb[q] + 1;
        const int64_t wd = S.super[d + 1] - S.super[d];
        chunks = std::max<int64_t>(chunks, ((m + 127) / 128 + (nc + 127) / 128) * ((wd + 31) / 32));
      }
      if (chunks > 0) NQG_CUDA(cudaMalloc(&P.d_wide_pack, (size_t)chunks * 32768));
      if (P.pers_map_ints > 0) NQG_CUDA(cudaMalloc(&P.d_pers_map, (size_t)P.pers_map_ints * sizeof(int)));
    }
    // control block: grid barriers of the blocked factorization, abort flag
    // of the block solves
    NQG_CUDA(cudaMalloc(&P.d_wide_ctl, wide_ctl_bytes()));
    NQG_CUDA(cudaMemset(P.d_wide_ctl, 0, wide_ctl_bytes()));
  }
  return NQG_OK;
}

static void free_plan(Plan &P) {
  void *ptrs[] = {P.d_super, P.d_col2sup, P.d_ls, P.d_ls_sym, P.d_lpi, P.d_lpx, P.d_Kp, P.d_Ki, P.d_Kx,
                  P.d_Rp, P.d_Rj, P.d_Rx, P.d_map_lo, P.d_map_hi, P.d_Kx_spmv, P.d_perm, P.d_iperm, P.d_locperm,
                  P.d_perm_tmp, P.d_L, P.d_D, P.d_tiles, P.d_tile_list, P.d_targets, P.d_pair_s, P.d_pair_d,
                  P.d_pair_lb, P.d_pair_ub, P.d_targets_lv, P.d_pivoted, P.d_visible, P.d_hidden, P.d_status,
                  P.d_xo, P.d_bo, P.d_r, P.d_w, P.d_in, P.d_out, P.d_V, P.d_scal, P.d_wide_W, P.d_wide_ctl,
                  P.d_wide_pack, P.d_pers_map, P.d_pair_map, P.d_pair_moff, P.d_map_items, P.d_locinv, P.d_pair_roff, P.d_rr_dest, P.d_rr_moved, P.d_rr_items, P.d_rr_stage,
                  P.d_solve_flags, P.d_xw, P.d_tinv, P.d_blk_items, P.d_flagoff, P.d_xf, P.d_Z, P.d_tiles_tc,
                  P.d_tile_list_tc, P.d_row_items};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  P.prof_collect();
  for (cudaEvent_t e : P.ev_pool) cudaEventDestroy(e);
  if (P.ev0) cudaEventDestroy(P.ev0);
  if (P.ev1) cudaEventDestroy(P.ev1);
  if (P.own_stream) cudaStreamDestroy(P.own_stream);
}

// Diagonal perturbation of the factored matrix.  regularization 1
// (reference find_perturbation, src/QP/linear_solver_wrapper.cpp:352-363):
// tiny diagonals become reg_diag, and the refinement matrix sees 0 there
// (set_diags(0), :1524-1533).  regularization 0 (apply_perturbation,
// :365-372): +reg_diag on the leading perturb_plus_cols diagonals, -reg_diag
// on the rest, and the refinement matrix keeps the unperturbed values
// (remove_perturbation before the refinement, :1362).  Every column's first
// stored entry is its diagonal (checked at plan creation).
static void apply_perturbation(Plan &P) {
  P.pert_idx.clear();
  P.Kx_spmv = P.K.x;
  if (P.set.regularization == 1) {
    for (int j = 0; j < P.n; ++j) {
      int q = P.K.p[j];
      if (q >= P.K.p[j + 1]) continue;
      if (std::abs(P.K.x[q]) < P.set.reg_diag) {
        P.K.x[q] = P.set.reg_diag;
        P.Kx_spmv[q] = 0.0;
        P.pert_idx.push_back(q);
      }
    }
  } else if (P.set.reg_diag != 0.0) {
    const int plus = P.set.perturb_plus_cols < 0 ? P.n : std::min(P.set.perturb_plus_cols, P.n);
    for (int j = 0; j < P.n; ++j) {
      int q = P.K.p[j];
      if (q >= P.K.p[j + 1]) continue;
      P.K.x[q] += j < plus ? P.set.reg_diag : -P.set.reg_diag;
    }
  }
  // FP32 factor: a larger, sign-keeping floor on the diagonal of the matrix
  // that is factored.  Pivots as small as the reference's 1e-8..1e-9
  // regularization create element growth of 1e8..1e9 under block-restricted
  // Bunch-Kaufman, beyond what FP32 values can carry; the refinement matrix
  // (Kx_spmv) is left as the reference defines it.
  if (P.set.precision == NQG_FP32) {
    double tau = P.set.reg_diag_fp32;
    if (tau <= 0) {
      double amax = 0;
      for (double v : P.Kx_spmv) amax = std::max(amax, std::abs(v));
      tau = 3e-5 * (amax > 0 ? amax : 1.0);
    }
    P.reg32 = tau;
    for (int j = 0; j < P.n; ++j) {
      int q = P.K.p[j];
      if (q >= P.K.p[j + 1]) continue;
      double v = P.K.x[q];
      if (std::abs(v) < tau) P.K.x[q] = v < 0 ? -tau : tau;
    }
  }
}

extern "C" int nqg_plan_create(int n, const int *Ap, const int *Ai, const double *Ax, const int *extra_cols,
                               const nqg_settings *settings, nqg_plan **out) {
  if (!out || !check_lower_csc(n, Ap, Ai) || (n > 0 && !Ax)) return NQG_ERR_ARG;
  *out = nullptr;
  auto *h = new (std::nothrow) nqg_plan;
  if (!h) return NQG_ERR_SIZE;
  Plan &P = h->P;
  if (settings) P.set = *settings;
  else nqg_default_settings(&P.set);
  // the refinement keeps its Hessenberg solution in 48 device scalar slots
  if (P.set.precision != NQG_FP64 && P.set.precision != NQG_FP32 ||
      (P.set.solve_precision != NQG_FP64 && P.set.solve_precision != NQG_FP32) || P.set.max_inner_iter > 48 ||
      P.set.max_inner_iter < 0 || P.set.req_ref_iter < 0) {
    delete h;
    return NQG_ERR_ARG;
  }
  P.n = n;
  P.K.n = n;
  P.K.p.assign(Ap, Ap + n + 1);
  P.K.i.assign(Ai, Ai + Ap[n]);
  P.K.x.assign(Ax, Ax + Ap[n]);
  apply_perturbation(P);
  std::string err = analyze(P.K, extra_cols, P.set.n_relax, P.set.z_relax, P.sym);
  if (!err.empty()) {
    P.last_error = err;
    delete h;
    return NQG_ERR_SYMBOLIC;
  }
  {
    Csc pat = P.K;
    pat.x.clear();
    sym_permute(pat, P.sym.iperm, nullptr, &P.Uord);
  }
  build_schedule(P);
  int rc = upload_plan(P);
  if (rc) {
    free_plan(P);
    delete h;
    return rc;
  }
  *out = h;
  return NQG_OK;
}

extern "C" int nqg_plan_destroy(nqg_plan *h) {
  if (!h) return NQG_ERR_ARG;
  free_plan(h->P);
  delete h;
  return NQG_OK;
}

extern "C" int nqg_set_stream(nqg_plan *h, void *stream) {
  if (!h) return NQG_ERR_ARG;
  h->P.stream = stream ? (cudaStream_t)stream : h->P.own_stream;
  return NQG_OK;
}

extern "C" int nqg_get_symbolic(const nqg_plan *h, const nqg_symbolic **sym) {
  if (!h || !sym) return NQG_ERR_ARG;
  // nqg_symbolic is layout-compatible with its single Symbolic member
  *sym = reinterpret_cast<const nqg_symbolic *>(&h->P.sym);
  return NQG_OK;
}

namespace {
// Refinement matrix values: CSC value q of the lower triangle goes to its
// position(s) in the full CSR (the pattern never changes).
__global__ void k_scatter_full(int64_t nz, const int64_t *mlo, const int64_t *mhi, const double *xv, double *Rx) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nz; q += (int64_t)gridDim.x * blockDim.x) {
    const double v = xv[q];
    Rx[mlo[q]] = v;
    if (mhi[q] >= 0) Rx[mhi[q]] = v;
  }
}
}  // namespace

extern "C" int nqg_set_values(nqg_plan *h, const double *Ax) {
  if (!h || (!Ax && h->P.n > 0)) return NQG_ERR_ARG;
  Plan &P = h->P;
  // the host copies below overwrite buffers that earlier copies read from
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  P.K.x.assign(Ax, Ax + P.K.nnz());
  apply_perturbation(P);
  const int64_t nz = (int64_t)P.K.nnz();
  NQG_CUDA(cudaMemcpyAsync(P.d_Kx, P.K.x.data(), nz * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  if (nz > 0) {
    if (!P.d_Kx_spmv) NQG_CUDA(cudaMalloc(&P.d_Kx_spmv, nz * sizeof(double)));
    NQG_CUDA(cudaMemcpyAsync(P.d_Kx_spmv, P.Kx_spmv.data(), nz * sizeof(double), cudaMemcpyHostToDevice, P.stream));
    k_scatter_full<<<(int)std::min<int64_t>((nz + 255) / 256, 4096), 256, 0, P.stream>>>(nz, P.d_map_lo, P.d_map_hi,
                                                                                          P.d_Kx_spmv, P.d_Rx);
    P.nlaunch++;
    NQG_CUDA(cudaGetLastError());
  }
  P.factored = false;
  return NQG_OK;
}

namespace {
__global__ void k_edit(int count, const int64_t *idx, const double *vals, const int64_t *mlo, const int64_t *mhi,
                       double *Kx, double *Rx) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    int64_t q = idx[t];
    double v = vals[t];
    Kx[q] = v;
    Rx[mlo[q]] = v;
    if (mhi[q] >= 0) Rx[mhi[q]] = v;
  }
}
}  // namespace

extern "C" int nqg_edit_values(nqg_plan *h, int count, const int64_t *idx, const double *vals) {
  if (!h || count < 0 || (count > 0 && (!idx || !vals))) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (count == 0) return NQG_OK;
  std::vector<double> kv(count), rv(count);
  for (int t = 0; t < count; ++t) {
    if (idx[t] < 0 || idx[t] >= P.K.nnz()) return NQG_ERR_ARG;
    P.K.x[idx[t]] = vals[t];
    P.Kx_spmv[idx[t]] = vals[t];
  }
  // staging: indices then values in the refinement workspace
  int64_t *d_idx = reinterpret_cast<int64_t *>(P.d_w);
  double *d_vals = P.d_r;
  if ((size_t)count > (size_t)std::max(P.n, 1)) return NQG_ERR_SIZE;
  NQG_CUDA(cudaMemcpyAsync(d_idx, idx, count * sizeof(int64_t), cudaMemcpyHostToDevice, P.stream));
  NQG_CUDA(cudaMemcpyAsync(d_vals, vals, count * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  k_edit<<<std::min((count + 255) / 256, 1024), 256, 0, P.stream>>>(count, d_idx, d_vals, P.d_map_lo, P.d_map_hi,
                                                                     P.d_Kx, P.d_Rx);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  return NQG_OK;
}

static int finish_factor(Plan &P) {
  int st = 0;
  NQG_CUDA(cudaMemcpyAsync(&st, P.d_status, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, P.ev0, P.ev1);
  P.tm.factor_ms = ms;
  if (st & ST_BOUNDS) {
    P.last_error = "device index check failed during factorization";
    return NQG_ERR_STATE;
  }
  if (st & ST_TIMEOUT) return NQG_ERR_TIMEOUT;
  P.factored = true;
  // a singular pivot block comes first: the non-finite values that follow
  // from it (divisions by its zero D entry) are its consequence
  if (st & ST_ZERO_PIVOT) return NQG_WARN_ZERO_PIVOT;
  if (st & ST_NONFINITE) return NQG_WARN_NONFINITE;
  return NQG_OK;
}

extern "C" int nqg_factor(nqg_plan *h) {
  if (!h) return NQG_ERR_ARG;
  Plan &P = h->P;
  NQG_CUDA(cudaMemsetAsync(P.d_status, 0, sizeof(int), P.stream));
  NQG_CUDA(cudaEventRecord(P.ev0, P.stream));
  int rc = dev_factor(P, nullptr);
  if (rc < 0) return rc;
  NQG_CUDA(cudaEventRecord(P.ev1, P.stream));
  return finish_factor(P);
}

extern "C" int nqg_refactor(nqg_plan *h, int count, const int *snodes) {
  if (!h || count < 0 || (count > 0 && !snodes)) return NQG_ERR_ARG;
  Plan &P = h->P;
  std::vector<int> sub(snodes, snodes + count);
  NQG_CUDA(cudaMemsetAsync(P.d_status, 0, sizeof(int), P.stream));
  NQG_CUDA(cudaEventRecord(P.ev0, P.stream));
  int rc = dev_factor(P, &sub);
  if (rc < 0) return rc;
  NQG_CUDA(cudaEventRecord(P.ev1, P.stream));
  return finish_factor(P);
}

extern "C" int nqg_set_visibility(nqg_plan *h, const uint8_t *visible_sn, const uint8_t *hidden_col) {
  if (!h) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!visible_sn && !hidden_col) {
    P.masked = false;
    return NQG_OK;
  }
  const int ns = P.sym.nsuper;
  std::vector<uint8_t> vis(ns, 1), hid(P.n, 0);
  if (visible_sn) std::copy(visible_sn, visible_sn + ns, vis.begin());
  if (hidden_col) std::copy(hidden_col, hidden_col + P.n, hid.begin());
  P.vis_host = vis;
  NQG_CUDA(cudaMemcpyAsync(P.d_visible, vis.data(), ns, cudaMemcpyHostToDevice, P.stream));
  NQG_CUDA(cudaMemcpyAsync(P.d_hidden, hid.data(), P.n, cudaMemcpyHostToDevice, P.stream));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  P.masked = true;
  return NQG_OK;
}

extern "C" int nqg_solve_device(nqg_plan *h, const double *d_rhs, double *d_x) {
  if (!h || !d_rhs || !d_x) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!P.factored) return NQG_ERR_STATE;
  NQG_CUDA(cudaEventRecord(P.ev0, P.stream));
  int rc = dev_solve(P, d_rhs, d_x);
  if (rc) return rc;
  NQG_CUDA(cudaEventRecord(P.ev1, P.stream));
  int st = 0;
  NQG_CUDA(cudaMemcpyAsync(&st, P.d_status, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
  NQG_CUDA(cudaEventSynchronize(P.ev1));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, P.ev0, P.ev1);
  P.tm.solve_ms = ms;
  if (st & ST_TIMEOUT) {  // a block-solve wait gave up: x is not a solution
    st &= ~ST_TIMEOUT;
    NQG_CUDA(cudaMemcpy(P.d_status, &st, sizeof(int), cudaMemcpyHostToDevice));
    P.last_error = "a cross-CTA wait of the triangular solves gave up";
    return NQG_ERR_TIMEOUT;
  }
  return NQG_OK;
}

extern "C" int nqg_set_wait_limit(nqg_plan *h, long long polls) {
  if (!h) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!P.d_wide_ctl) return NQG_ERR_STATE;
  const long long v = polls > 0 ? polls : 0;
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  NQG_CUDA(cudaMemcpy(static_cast<char *>(P.d_wide_ctl) + wide_ctl_limit_offset(), &v, sizeof(v),
                      cudaMemcpyHostToDevice));
  return NQG_OK;
}

extern "C" int nqg_solve(nqg_plan *h, const double *rhs, double *x) {
  if (!h || (!rhs && h->P.n > 0) || (!x && h->P.n > 0)) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!P.factored) return NQG_ERR_STATE;
  NQG_CUDA(cudaMemcpyAsync(P.d_in, rhs, P.n * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  int rc = nqg_solve_device(h, P.d_in, P.d_out);
  if (rc) return rc;
  NQG_CUDA(cudaMemcpyAsync(x, P.d_out, P.n * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  return NQG_OK;
}

extern "C" int nqg_refine_only(nqg_plan *h, const double *rhs, double *x) {
  if (!h || (!rhs && h->P.n > 0) || (!x && h->P.n > 0)) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!P.factored) return NQG_ERR_STATE;
  NQG_CUDA(cudaMemcpyAsync(P.d_in, rhs, P.n * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  NQG_CUDA(cudaEventRecord(P.ev0, P.stream));
  int rc = dev_refine_only(P, P.d_in, P.d_out);
  if (rc) return rc;
  NQG_CUDA(cudaEventRecord(P.ev1, P.stream));
  int st = 0;
  NQG_CUDA(cudaMemcpyAsync(&st, P.d_status, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
  NQG_CUDA(cudaMemcpyAsync(x, P.d_out, P.n * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, P.ev0, P.ev1);
  P.tm.solve_ms = ms;
  if (st & ST_TIMEOUT) {
    st &= ~ST_TIMEOUT;
    NQG_CUDA(cudaMemcpy(P.d_status, &st, sizeof(int), cudaMemcpyHostToDevice));
    P.last_error = "a cross-CTA wait of the triangular solves gave up";
    return NQG_ERR_TIMEOUT;
  }
  return NQG_OK;
}

extern "C" int nqg_ldlt_solve_ordered_device(nqg_plan *h, double *d_x_ord) {
  if (!h || !d_x_ord) return NQG_ERR_ARG;
  Plan &P = h->P;
  if (!P.factored) return NQG_ERR_STATE;
  return dev_ldlt_solve_ord(P, d_x_ord);
}

extern "C" int nqg_spmv_device(nqg_plan *h, const double *d_x, double *d_y) {
  if (!h || !d_x || !d_y) return NQG_ERR_ARG;
  return dev_spmv_orig(h->P, d_x, d_y);
}

// 2x2 pivot blocks (nonzero sub-diagonal entries of D) and supernodes that
// Bunch-Kaufman permuted in the last factorization; counts[0..1] on device.
template <class T>
__global__ void k_pivot_counts(int n, const T *Dg, int ns, const uint8_t *pivoted, int *counts) {
  int a = 0, b = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a += Dg[n + i] != T(0);
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) b += pivoted[s] != 0;
  if (a) atomicAdd(&counts[0], a);
  if (b) atomicAdd(&counts[1], b);
}

extern "C" int nqg_get_timings(const nqg_plan *h, nqg_timings *t) {
  if (!h || !t) return NQG_ERR_ARG;
  Plan &P = const_cast<nqg_plan *>(h)->P;
  if (P.factored) {
    // pivot statistics of the last factorization, counted on demand
    int *cnt = reinterpret_cast<int *>(P.d_scal + 60);  // spare slots of the scalar area
    NQG_CUDA(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), P.stream));
    const int blocks = std::max(1, std::min((P.n + 255) / 256, 1024));
    if (P.set.precision == NQG_FP32)
      k_pivot_counts<float><<<blocks, 256, 0, P.stream>>>(P.n, reinterpret_cast<const float *>(P.d_D),
                                                          P.sym.nsuper, P.d_pivoted, cnt);
    else
      k_pivot_counts<double><<<blocks, 256, 0, P.stream>>>(P.n, reinterpret_cast<const double *>(P.d_D),
                                                           P.sym.nsuper, P.d_pivoted, cnt);
    int hc[2] = {0, 0};
    NQG_CUDA(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, P.stream));
    NQG_CUDA(cudaStreamSynchronize(P.stream));
    P.tm.num_2x2 = hc[0];
    P.tm.num_pivot_supernodes = hc[1];
  }
  *t = P.tm;
  return NQG_OK;
}

extern "C" int nqg_get_factor(const nqg_plan *hc, double *values, double *d, int *perm, int *ls) {
  if (!hc) return NQG_ERR_ARG;
  Plan &P = const_cast<nqg_plan *>(hc)->P;
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  const int n = P.n;
  if (values) {
    if (P.set.precision == NQG_FP32) {
      std::vector<float> tmp(P.sym.xsize);
      NQG_CUDA(cudaMemcpy(tmp.data(), P.d_L, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < tmp.size(); ++q) values[q] = tmp[q];
    } else {
      NQG_CUDA(cudaMemcpy(values, P.d_L, (size_t)P.sym.xsize * sizeof(double), cudaMemcpyDeviceToHost));
    }
  }
  if (d) {
    if (P.set.precision == NQG_FP32) {
      std::vector<float> tmp(2 * n);
      NQG_CUDA(cudaMemcpy(tmp.data(), P.d_D, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < tmp.size(); ++q) d[q] = tmp[q];
    } else {
      NQG_CUDA(cudaMemcpy(d, P.d_D, (size_t)2 * n * sizeof(double), cudaMemcpyDeviceToHost));
    }
  }
  if (perm) NQG_CUDA(cudaMemcpy(perm, P.d_perm, n * sizeof(int), cudaMemcpyDeviceToHost));
  if (ls) NQG_CUDA(cudaMemcpy(ls, P.d_ls, P.ssize * sizeof(int), cudaMemcpyDeviceToHost));
  return NQG_OK;
}

extern "C" int nqg_get_device_status(const nqg_plan *hc, int *bits) {
  if (!hc || !bits) return NQG_ERR_ARG;
  Plan &P = const_cast<nqg_plan *>(hc)->P;
  NQG_CUDA(cudaMemcpy(bits, P.d_status, sizeof(int), cudaMemcpyDeviceToHost));
  return NQG_OK;
}

// ---- measurement -------------------------------------------------------------
namespace nqg {
cudaEvent_t Plan::prof_begin() {
  if (!prof) return nullptr;
  cudaEvent_t e;
  if (!ev_pool.empty()) {
    e = ev_pool.back();
    ev_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return nullptr;
  }
  cudaEventRecord(e, stream);
  return e;
}
void Plan::prof_end(int cls, cudaEvent_t a, double flops, double bytes) {
  if (!prof || !a) return;
  cudaEvent_t e;
  if (!ev_pool.empty()) {
    e = ev_pool.back();
    ev_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return;
  }
  cudaEventRecord(e, stream);
  prof_pending.push_back(ProfRec{cls, a, e, flops, bytes});
  if (prof_pending.size() > 8192 && !prof_hold) prof_collect();
}
void Plan::prof_collect() {
  if (prof_pending.empty()) return;
  cudaStreamSynchronize(stream);
  for (auto &r : prof_pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    auto &k = kstats[r.cls];
    k.launches += 1;
    k.total_ms += ms;
    k.alg_flops += r.flops;
    k.alg_bytes += r.bytes;
    ev_pool.push_back(r.a);
    ev_pool.push_back(r.b);
  }
  prof_pending.clear();
}
}  // namespace nqg

extern "C" int nqg_set_profiling(nqg_plan *h, int on) {
  if (!h) return NQG_ERR_ARG;
  Plan &P = h->P;
  P.prof_collect();
  P.prof = on != 0;
  for (auto &k : P.kstats) k = nqg_kernel_stats{};
  return NQG_OK;
}

extern "C" int nqg_get_kernel_stats(nqg_plan *h, int cls, nqg_kernel_stats *st) {
  if (!h || !st || cls < 0 || cls >= NQG_K_CLASSES) return NQG_ERR_ARG;
  h->P.prof_collect();
  *st = h->P.kstats[cls];
  return NQG_OK;
}

extern "C" int nqg_get_launch_count(const nqg_plan *h, long long *count) {
  if (!h || !count) return NQG_ERR_ARG;
  *count = h->P.nlaunch;
  return NQG_OK;
}
