// Supernodal LDL^T numeric factorization with Bunch-Kaufman pivoting inside
// each supernode's diagonal block, level-scheduled on one GPU.
//
// Per level of the supernodal assembly tree (leaves first):
//   1. k_update: every (target s, descendant d) Schur contribution
//      L_d D_d L_d^T restricted to s, tiled 64x64, accumulated in registers
//      and subtracted from s with atomics (reference left-looking loop,
//      src/ldl/Serial_blocked_ldl_02_2.cpp:69-129);
//   2. k_bk_*: Bunch-Kaufman on the diagonal block with explicit row swaps
//      (LAPACK dsytrf('L') + reorder_after_sytrf, Sym_BLAS.cpp:128-196),
//      then the panel column permutation (dlapmt), the unit triangular solve
//      with L11^T (dtrsm) and the D^-1 scaling (blocked_2by2_solver,
//      Sym_BLAS.cpp:492-529).
// After all levels, k_row_rename / k_row_move rename the rows of descendants
// that fall into pivoted supernodes and re-sort them (row_reordering,
// Sym_BLAS.cpp:327-490), and k_perm_compose folds the pivots into the global
// permutation (reorder_matrix, linear_solver_wrapper.cpp:1432-1460).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>

#include "plan.hpp"
#include "tcgen05.cuh"
#include "bk.cuh"

namespace nqg {

namespace {

constexpr int BK_THREADS = 128;
constexpr int UPD_THREADS = 256;
constexpr int UPD_KC = 16;

// ---------------------------------------------------------------------------
// k_zero_targets / k_assemble: reset the values of the supernodes being
// factored and scatter the (perturbed) matrix entries into them.
template <class T>
__global__ void k_zero_targets(const int *targets, int ntargets, const int *super, const int64_t *lpi,
                               const int64_t *lpx, T *L, T *D, int n) {
  const int s = targets[blockIdx.x];
  const int64_t beg = lpx[s], end = lpx[s + 1];
  for (int64_t q = beg + threadIdx.x; q < end; q += blockDim.x) L[q] = T(0);
  for (int c = super[s] + threadIdx.x; c < super[s + 1]; c += blockDim.x) {
    D[c] = T(0);
    D[n + c] = T(0);
  }
}

__device__ __forceinline__ int lower_bound_i(const int *a, int len, int key);

// Target row positions of the rows lb + r0 .. of descendant pair q (item
// (q, r0), one thread per row): row r of d goes to r - cs0 inside the
// target's diagonal block, else to its place in the target's row list.  The
// update tiles of the level read them instead of searching per tile.
__global__ void __launch_bounds__(256) k_pair_rowmap(const int2 *items, const int *pair_s, const int *pair_d,
                                                     const int *pair_lb, const int64_t *moff, const int *super,
                                                     const int64_t *lpi, const int *ls, int *map, int *status) {
  const int q = items[blockIdx.x].x, i = items[blockIdx.x].y + threadIdx.x;
  const int s = pair_s[q], d = pair_d[q], lb = pair_lb[q];
  const int m = (int)(lpi[d + 1] - lpi[d]) - lb;
  if (i >= m) return;
  const int r = ls[lpi[d] + lb + i];
  const int cs0 = super[s], ws = super[s + 1] - cs0;
  const int nrs = (int)(lpi[s + 1] - lpi[s]);
  const int *rows_s = ls + lpi[s];
  int pos;
  if (r < cs0 + ws) {
    pos = r - cs0;
  } else {
    pos = ws + lower_bound_i(rows_s + ws, nrs - ws, r);
    if (pos >= nrs || rows_s[pos] != r) {
      flag_status(status, ST_BOUNDS);
      pos = -1;
    }
  }
  map[moff[q] + i] = pos;
}

__device__ __forceinline__ int lower_bound_i(const int *a, int len, int key) {
  int lo = 0, hi = len;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <class T>
__global__ void k_assemble(int n, const int *Kp, const int *Ki, const double *Kx, const int *iperm, const int *col2sup,
                           const int *super, const int64_t *lpi, const int64_t *lpx, const int *ls, const uint8_t *mark,
                           T *L, int *status) {
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += warps) {
    const int bj = iperm[j];
    for (int q = Kp[j] + lane; q < Kp[j + 1]; q += 32) {
      const int bi = iperm[Ki[q]];
      const int c = min(bi, bj), r = max(bi, bj);
      const int s = col2sup[c];
      if (mark && !mark[s]) continue;
      const int c0 = super[s], w = super[s + 1] - c0;
      const int nrow = (int)(lpi[s + 1] - lpi[s]);
      int pos;
      if (r < c0 + w) {
        pos = r - c0;
      } else {
        const int *rows = ls + lpi[s] + w;
        pos = w + lower_bound_i(rows, nrow - w, r);
        if (pos >= nrow || ls[lpi[s] + pos] != r) {
          flag_status(status, ST_BOUNDS);
          continue;
        }
      }
      L[lpx[s] + (int64_t)(c - c0) * nrow + pos] = (T)Kx[q];
    }
  }
}

// ---------------------------------------------------------------------------
// Schur update tiles.  C = (L_d D_d)[rows] * L_d[cols]^T, subtracted from the
// target with atomics.  D_d is block diagonal with 1x1 and 2x2 blocks:
// (L D)(:,t) = d_t L(:,t) + e_t L(:,t+1) + e_{t-1} L(:,t-1) with e the 2x2
// sub-diagonals (zero outside 2x2 blocks), which is blocked_2by2_mult.
template <class T>
__global__ void __launch_bounds__(UPD_THREADS) k_update(const UpdTile *tiles, const int *tile_ids, int ntiles, int n,
                                                       const int *super, const int64_t *lpi, const int64_t *lpx,
                                                       const int *ls, T *L, const T *Dg, int *status,
                                                       const int *rowmap, const int64_t *pmoff, const int *pair_lb) {
  __shared__ T As[UPD_KC][UPD_TM + 1];
  __shared__ T Bs[UPD_KC][UPD_TN + 1];
  __shared__ T Raw[UPD_KC + 2][UPD_TM + 1];
  __shared__ T dk[UPD_KC + 2], ek[UPD_KC + 2];
  __shared__ int prow[UPD_TM], pcol[UPD_TN];
  const int tid = threadIdx.x;
  const UpdTile tl = tiles[tile_ids ? tile_ids[blockIdx.x] : blockIdx.x];
  const int s = tl.s, d = tl.d;
  const int c0 = super[d], wd = super[d + 1] - c0;
  const int nrd = (int)(lpi[d + 1] - lpi[d]);
  const int *rows_d = ls + lpi[d];
  const T *Ld = L + lpx[d];
  const int mrows = min(UPD_TM, nrd - tl.ri);
  const int ncols = min(UPD_TN, tl.ub + 1 - tl.cj);
  const int cs0 = super[s], ws = super[s + 1] - cs0;
  const int nrs = (int)(lpi[s + 1] - lpi[s]);
  T *Lt = L + lpx[s];
  // target positions of the tile's rows (from the level's pair map) and columns
  const int *pmap = rowmap + pmoff[tl.q] + (tl.ri - pair_lb[tl.q]);
  for (int i = tid; i < UPD_TM; i += blockDim.x) prow[i] = i < mrows ? pmap[i] : -1;
  for (int j = tid; j < UPD_TN; j += blockDim.x) {
    int pos = -1;
    if (j < ncols) {
      pos = rows_d[tl.cj + j] - cs0;
      if (pos < 0 || pos >= ws) {
        flag_status(status, ST_BOUNDS);
        pos = -1;
      }
    }
    pcol[j] = pos;
  }
  const int tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
  for (int t0 = 0; t0 < wd; t0 += UPD_KC) {
    __syncthreads();
    // raw columns t0-1 .. t0+KC of the tile rows, plus D entries
    for (int e = tid; e < (UPD_KC + 2) * UPD_TM; e += blockDim.x) {
      int cc = e / UPD_TM, i = e % UPD_TM;
      int t = t0 - 1 + cc;
      T v = T(0);
      if (t >= 0 && t < wd && i < mrows) v = Ld[(size_t)t * nrd + tl.ri + i];
      Raw[cc][i] = v;
    }
    for (int cc = tid; cc < UPD_KC + 2; cc += blockDim.x) {
      int t = t0 - 1 + cc;
      dk[cc] = (t >= 0 && t < wd) ? Dg[c0 + t] : T(0);
      ek[cc] = (t >= 0 && t < wd) ? Dg[n + c0 + t] : T(0);
    }
    for (int e = tid; e < UPD_KC * UPD_TN; e += blockDim.x) {
      int cc = e / UPD_TN, j = e % UPD_TN;
      int t = t0 + cc;
      Bs[cc][j] = (t < wd && j < ncols) ? Ld[(size_t)t * nrd + tl.cj + j] : T(0);
    }
    __syncthreads();
    for (int e = tid; e < UPD_KC * UPD_TM; e += blockDim.x) {
      int cc = e / UPD_TM, i = e % UPD_TM;
      // column t = t0+cc sits at Raw index cc+1
      As[cc][i] = dk[cc + 1] * Raw[cc + 1][i] + ek[cc + 1] * Raw[cc + 2][i] + ek[cc] * Raw[cc][i];
    }
    __syncthreads();
#pragma unroll
    for (int cc = 0; cc < UPD_KC; ++cc) {
      T av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[cc][ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = Bs[cc][tx * 4 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = ty * 4 + a;
    if (i >= mrows || prow[i] < 0) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = tx * 4 + b;
      if (j >= ncols || pcol[j] < 0) continue;
      if (tl.ri + i < tl.cj + j) continue;  // lower part only
      atomicAdd(&Lt[(size_t)pcol[j] * nrs + prow[i]], -acc[a][b]);
    }
  }
}

// FP32 Schur update tiles of 128 x 128 on the fifth-generation tensor cores
// (descendants of UPD_TC_MIN_WD or more columns): the same (L_d D_d)[rows] *
// L_d[cols]^T as k_update, with the D_d product applied while the rows of the
// A operand are loaded, split-TF32 products accumulated in TMEM, and the
// atomic scatter into the target from the TMEM rows (thread r owns row r).
__global__ void __launch_bounds__(t5::THREADS) k_update_t5(const UpdTile *tiles, const int *tile_ids, int n,
                                                           const int *super, const int64_t *lpi, const int64_t *lpx,
                                                           const int *ls, float *L, const float *Dg, int *status,
                                                           const int *rowmap, const int64_t *pmoff,
                                                           const int *pair_lb) {
  extern __shared__ __align__(1024) unsigned char t5_smem[];
  __shared__ int prow[UPD_TC_T], pcol[UPD_TC_T];
  const int tid = threadIdx.x;
  const UpdTile tl = tiles[tile_ids[blockIdx.x]];
  const int s = tl.s, d = tl.d;
  const int c0 = super[d], wd = super[d + 1] - c0;
  const int nrd = (int)(lpi[d + 1] - lpi[d]);
  const int *rows_d = ls + lpi[d];
  const float *Ld = L + lpx[d];
  const int mrows = min(UPD_TC_T, nrd - tl.ri);
  const int ncols = min(UPD_TC_T, tl.ub + 1 - tl.cj);
  const int cs0 = super[s], ws = super[s + 1] - cs0;
  const int nrs = (int)(lpi[s + 1] - lpi[s]);
  float *Lt = L + lpx[s];
  {
    // target positions of row tid (from the level's pair map) and column tid
    int pos = tid < mrows ? rowmap[pmoff[tl.q] + (tl.ri - pair_lb[tl.q]) + tid] : -1;
    prow[tid] = pos;
    pos = -1;
    if (tid < ncols) {
      pos = rows_d[tl.cj + tid] - cs0;
      if (pos < 0 || pos >= ws) {
        flag_status(status, ST_BOUNDS);
        pos = -1;
      }
    }
    pcol[tid] = pos;
  }
  __syncthreads();
  const float *Dd = Dg + c0, *Ed = Dg + n + c0;
  // row r of L_d D_d: column t is d_t L(:,t) + e_t L(:,t+1) + e_{t-1} L(:,t-1)
  auto fa = [&](int r, int k0, float(&x)[t5::TK]) {
    const bool ok = r < mrows;
    const float *Lr = Ld + tl.ri + r;
    float raw[t5::TK + 2];
#pragma unroll
    for (int q = 0; q < t5::TK + 2; ++q) {
      const int t = k0 - 1 + q;
      raw[q] = (ok && t >= 0 && t < wd) ? Lr[(size_t)t * nrd] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < t5::TK; ++k) {
      const int t = k0 + k;
      const float dk = t < wd ? Dd[t] : 0.f, ek = t < wd ? Ed[t] : 0.f;
      const float em = (t >= 1 && t - 1 < wd) ? Ed[t - 1] : 0.f;
      x[k] = dk * raw[k + 1] + ek * raw[k + 2] + em * raw[k];
    }
  };
  auto fb = [&](int c, int k0, float(&x)[t5::TK]) {
    const bool ok = c < ncols;
    const float *Lc = Ld + tl.cj + c;
#pragma unroll
    for (int k = 0; k < t5::TK; ++k) x[k] = (ok && k0 + k < wd) ? Lc[(size_t)(k0 + k) * nrd] : 0.f;
  };
  auto ep = [&](int r, int cb, const uint32_t(&v)[32]) {
    if (r >= mrows || prow[r] < 0) return;
    float *dst = Lt + prow[r];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int c = cb + q;
      if (c < ncols && pcol[c] >= 0 && tl.ri + r >= tl.cj + c)
        atomicAdd(dst + (size_t)pcol[c] * nrs, -__uint_as_float(v[q]));
    }
  };
  t5::tile_tf32x3<1>(wd, fa, fb, ep, t5_smem, status);
}

// ---------------------------------------------------------------------------
// Diagonal block BK + panel, one CTA per supernode.  SMALL: the block and a
// row chunk of the panel are staged in shared memory.
template <class T>
__global__ void __launch_bounds__(BK_THREADS) k_bk_small(const int *targets, int n, const int *super,
                                                         const int64_t *lpi, const int64_t *lpx, T *L, T *Dg,
                                                         int *locperm, uint8_t *pivoted, int *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *a = reinterpret_cast<T *>(smem_raw);                 // BK_SMALL * BK_SMALL
  T *rowbuf = a + BK_SMALL * BK_SMALL;                     // BK_SMALL * BK_THREADS
  __shared__ int perm[BK_SMALL];
  const int s = targets[blockIdx.x];
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  T *Ls = L + lpx[s];
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    int c = e / w, r = e % w;
    a[r + c * w] = r >= c ? Ls[r + (size_t)c * nrow] : T(0);
  }
  __syncthreads();
  bool piv = false;
  bk_factor(a, w, w, Dg + c0, Dg + n + c0, perm, status, &piv);
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    int c = e / w, r = e % w;
    Ls[r + (size_t)c * nrow] = r >= c ? a[r + c * w] : T(0);
  }
  for (int m = threadIdx.x; m < w; m += blockDim.x) locperm[c0 + m] = perm[m];
  if (threadIdx.x == 0) pivoted[s] = piv ? 1 : 0;
  __syncthreads();
  panel_solve_rows(Ls, nrow, w, a, w, Dg + c0, Dg + n + c0, perm, rowbuf, BK_THREADS, piv);
  // non-finite check on D
  bool bad = false;
  for (int m = threadIdx.x; m < w; m += blockDim.x) {
    T v = Dg[c0 + m];
    if (!isfinite((double)v)) bad = true;
  }
  if (block_any(bad) && threadIdx.x == 0) flag_status(status, ST_NONFINITE);
}

// GENERIC: the diagonal block is factored in place in global memory; the
// panel is permuted in place by following the permutation's cycles and
// solved one row per thread.
template <class T>
__global__ void __launch_bounds__(256) k_bk_global(const int *targets, int n, const int *super, const int64_t *lpi,
                                                   const int64_t *lpx, T *L, T *Dg, int *locperm, uint8_t *pivoted,
                                                   int *cycle_buf, int do_rows, int *status, int staged) {
  extern __shared__ __align__(16) unsigned char bkg_raw[];
  const int s = targets[blockIdx.x];
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  T *Ls = L + lpx[s];
  int *perm = locperm + c0;
  bool piv = false;
  if (staged) {
    // the whole diagonal block in shared memory (staged: the launch's
    // dynamic shared memory holds w x w values), factored there, written back
    T *a = reinterpret_cast<T *>(bkg_raw);
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int c = e / w, r = e % w;
      a[e] = r >= c ? Ls[r + (size_t)c * nrow] : T(0);
    }
    __syncthreads();
    bk_factor(a, w, w, Dg + c0, Dg + n + c0, perm, status, &piv);
    __syncthreads();
    // strict upper triangle back to 0 (never referenced, kept at 0 like the reference)
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int c = e / w, r = e % w;
      Ls[r + (size_t)c * nrow] = r >= c ? a[e] : T(0);
    }
  } else {
    bk_factor(Ls, nrow, w, Dg + c0, Dg + n + c0, perm, status, &piv);
    // zero the strict upper triangle (never referenced, kept at 0 like the reference)
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      int c = e / w, r = e % w;
      if (r < c) Ls[r + (size_t)c * nrow] = T(0);
    }
  }
  if (threadIdx.x == 0) pivoted[s] = piv ? 1 : 0;
  __syncthreads();
  const T *D = Dg + c0, *E = Dg + n + c0;
  // cycle leaders of the column permutation new[j] = old[perm[j]]
  int *lead = cycle_buf + c0;  // n-sized scratch, this supernode's slice
  if (piv && do_rows) {
    for (int j = threadIdx.x; j < w; j += blockDim.x) {
      // j leads its cycle if it is the smallest index on it
      int q = perm[j], isl = 1;
      int guard = 0;
      while (q != j && guard++ <= w) {
        if (q < j) {
          isl = 0;
          break;
        }
        q = perm[q];
      }
      lead[j] = isl;
    }
  }
  __syncthreads();
  for (int r = w + threadIdx.x; do_rows && r < nrow; r += blockDim.x) {
    T *row = Ls + r;  // element j at row[j*nrow]
    if (piv) {
      for (int j = 0; j < w; ++j) {
        if (!lead[j] || perm[j] == j) continue;
        // new[j] = old[perm[j]]: rotate along the cycle starting at j
        T first = row[(size_t)j * nrow];
        int cur = j, guard = 0;
        while (guard++ <= w) {
          int nx = perm[cur];
          if (nx == j) {
            row[(size_t)cur * nrow] = first;
            break;
          }
          row[(size_t)cur * nrow] = row[(size_t)nx * nrow];
          cur = nx;
        }
      }
    }
    for (int j = 0; j < w; ++j) {
      T x = row[(size_t)j * nrow];
      for (int t = 0; t < j; ++t) x -= row[(size_t)t * nrow] * Ls[j + (size_t)t * nrow];
      row[(size_t)j * nrow] = x;
    }
    for (int j = 0; j < w; ++j) {
      if (E[j] == T(0)) {
        T inv = T(1) / D[j];
        row[(size_t)j * nrow] *= inv;
      } else {
        T sd = E[j];
        T det = D[j] * D[j + 1] - sd * sd;
        T inv = T(1) / det;
        T x1 = row[(size_t)j * nrow], x2 = row[(size_t)(j + 1) * nrow];
        row[(size_t)j * nrow] = (x1 * D[j + 1] - x2 * sd) * inv;
        row[(size_t)(j + 1) * nrow] = (x2 * D[j] - x1 * sd) * inv;
        ++j;
      }
    }
  }
  bool bad = false;
  for (int m = threadIdx.x; m < w; m += blockDim.x)
    if (!isfinite((double)D[m])) bad = true;
  if (block_any(bad) && threadIdx.x == 0) flag_status(status, ST_NONFINITE);
}

// ---------------------------------------------------------------------------
// Rows below the diagonal block of a supernode factored by k_bk_global:
// L21 = (A21 P^T) L11^-T D^-1 (dlapmt + dtrsm + blocked_2by2_solver,
// src/ldl/Serial_blocked_ldl_02_2.cpp:137-161), spread over (supernode,
// 64-row block) items.  The CTA stages its rows with the pivot column order
// applied, then works through L11 in panels of PR_KB columns staged in shared
// memory: each panel's triangle is solved one row per thread, and its
// contribution is subtracted from the later columns.  Every entry receives
// the terms x_t L(j, t) in increasing t, as in the per-row substitution.
constexpr int PR_ROWS = 64, PR_KB = 32, PR_CG = 4;  // rows per item, panel width, columns per thread

__host__ __device__ constexpr size_t panel_rows_smem(int wmax, int vsize) {
  return ((size_t)PR_ROWS * (wmax + 1) + (size_t)wmax * (PR_KB + 1)) * vsize;
}

template <class T>
__global__ void __launch_bounds__(256) k_panel_rows(const int2 *items, int n, const int *super, const int64_t *lpi,
                                                    const int64_t *lpx, T *L, const T *Dg, const int *locperm,
                                                    const uint8_t *pivoted) {
  extern __shared__ __align__(16) unsigned char pr_raw[];
  const int s = items[blockIdx.x].x, rb = items[blockIdx.x].y;
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  T *Ls = L + lpx[s];
  const int *perm = locperm + c0;
  const bool piv = pivoted[s] != 0;
  const int r0 = w + rb * PR_ROWS, m = min(PR_ROWS, nrow - r0);
  if (m <= 0) return;
  const int ldx = w + 1;
  T *X = reinterpret_cast<T *>(pr_raw);  // [PR_ROWS][ldx]
  T *Lp = X + (size_t)PR_ROWS * ldx;     // [w][PR_KB + 1]: columns jb .. jb+kb of L11, rows jb .. w
  const int tid = threadIdx.x;
  for (int e = tid; e < m * w; e += blockDim.x) {
    const int r = e % m, j = e / m;
    X[r * ldx + j] = Ls[(r0 + r) + (size_t)(piv ? perm[j] : j) * nrow];
  }
  for (int jb = 0; jb < w; jb += PR_KB) {
    const int kb = min(PR_KB, w - jb);
    __syncthreads();
    for (int e = tid; e < (w - jb) * kb; e += blockDim.x) {
      const int i = e % (w - jb), jj = e / (w - jb);
      Lp[i * (PR_KB + 1) + jj] = Ls[(jb + i) + (size_t)(jb + jj) * nrow];
    }
    __syncthreads();
    // triangle of the panel: row r, columns jb .. jb+kb
    if (tid < m) {
      T *xr = X + tid * ldx;
      for (int j = 0; j < kb; ++j) {
        T x = xr[jb + j];
        for (int t = 0; t < j; ++t) x -= xr[jb + t] * Lp[j * (PR_KB + 1) + t];
        xr[jb + j] = x;
      }
    }
    __syncthreads();
    // later columns c >= jb+kb: x(r, c) -= sum_t x(r, jb+t) L(c, jb+t), t increasing
    const int c_lo = jb + kb, ncg = (w - c_lo + PR_CG - 1) / PR_CG;
    for (int e = tid; e < m * ncg; e += blockDim.x) {
      const int r = e % m, cg0 = c_lo + (e / m) * PR_CG;
      T *xr = X + r * ldx;
      T acc[PR_CG];
#pragma unroll
      for (int q = 0; q < PR_CG; ++q) acc[q] = cg0 + q < w ? xr[cg0 + q] : T(0);
      for (int t = 0; t < kb; ++t) {
        const T xt = xr[jb + t];
#pragma unroll
        for (int q = 0; q < PR_CG; ++q)
          if (cg0 + q < w) acc[q] -= xt * Lp[(cg0 + q - jb) * (PR_KB + 1) + t];
      }
#pragma unroll
      for (int q = 0; q < PR_CG; ++q)
        if (cg0 + q < w) xr[cg0 + q] = acc[q];
    }
  }
  __syncthreads();
  // D^-1 (1x1 and 2x2 blocks, Cramer's rule) and write back
  const T *D = Dg + c0, *E = Dg + n + c0;
  if (tid < m) {
    T *xr = X + tid * ldx;
    for (int j = 0; j < w; ++j) {
      if (E[j] == T(0)) {
        T inv = T(1) / D[j];
        xr[j] *= inv;
      } else {
        T sd = E[j];
        T det = D[j] * D[j + 1] - sd * sd;
        T inv = T(1) / det;
        T x1 = xr[j], x2 = xr[j + 1];
        xr[j] = (x1 * D[j + 1] - x2 * sd) * inv;
        xr[j + 1] = (x2 * D[j] - x1 * sd) * inv;
        ++j;
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < m * w; e += blockDim.x) {
    const int r = e % m, j = e / m;
    Ls[(r0 + r) + (size_t)j * nrow] = X[r * ldx + j];
  }
}

// ---------------------------------------------------------------------------
// Row renaming after pivoting (row_reordering, Sym_BLAS.cpp:327-490): for a
// (pivoted target s, descendant d) pair, the rows of d in s's column range
// [lb, ub] are renamed through s's inverse pivot order and re-sorted, and
// d's value rows move along.  Three launches, each O(rows) per pair:
//   k_loc_inverse  locinv[c0 + locperm[c0 + m]] = m for pivoted supernodes;
//   k_row_rename   one warp per pair: new names, their ranks (a bitmap over
//                  s's columns + prefix popcounts) = the new positions,
//                  sorted names written back, positions kept in dest;
//   k_row_move     (pair, column chunk) items: the chunk's rows staged in
//                  shared memory (global scratch for very long runs), then
//                  stored at their new positions.

__global__ void k_loc_inverse(int n, const int *col2sup, const int *super, const uint8_t *pivoted,
                              const int *locperm, int *locinv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = col2sup[i];
    if (!pivoted[s]) continue;
    const int c0 = super[s];
    locinv[c0 + locperm[i]] = i - c0;
  }
}

__global__ void k_row_rename(const int *pair_s, const int *pair_d, const int *pair_lb, const int *pair_ub,
                             int64_t npairs, const int64_t *pair_roff, const uint8_t *pivoted, const int *super,
                             const int64_t *lpi, int *ls, const int *locinv, int *dest_all, uint8_t *moved,
                             int words_per_warp, int *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t p = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (p >= npairs) return;
  const int s = pair_s[p];
  if (!pivoted[s]) {
    if (lane == 0) moved[p] = 0;
    return;
  }
  const int d = pair_d[p], lb = pair_lb[p];
  const int len = pair_ub[p] - lb + 1;
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nwords = (w + 31) >> 5;
  unsigned *bits = reinterpret_cast<unsigned *>(smem_raw) + (size_t)warp * 2 * words_per_warp;
  unsigned *wpre = bits + words_per_warp;
  int *rows = ls + lpi[d] + lb;
  int *dest = dest_all + pair_roff[p];
  for (int q = lane; q < nwords; q += 32) bits[q] = 0u;
  __syncwarp();
  for (int e = lane; e < len; e += 32) {
    int r = rows[e] - c0;
    int nw = (r >= 0 && r < w) ? locinv[c0 + r] : -1;
    if (nw < 0 || nw >= w) {
      flag_status(status, ST_BOUNDS);
      nw = 0;
    }
    dest[e] = nw;
    atomicOr(&bits[nw >> 5], 1u << (nw & 31));
  }
  __syncwarp();
  // exclusive prefix of the word popcounts: contiguous segments per lane
  const int seg = (nwords + 31) >> 5;
  const int q0 = min(lane * seg, nwords), q1 = min(q0 + seg, nwords);
  unsigned cnt = 0;
  for (int q = q0; q < q1; ++q) cnt += __popc(bits[q]);
  unsigned incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  unsigned acc = incl - cnt;
  for (int q = q0; q < q1; ++q) {
    wpre[q] = acc;
    acc += __popc(bits[q]);
  }
  __syncwarp();
  int mv = 0;
  for (int e = lane; e < len; e += 32) {
    const int nw = dest[e];
    const int rank = (int)(wpre[nw >> 5] + __popc(bits[nw >> 5] & ((1u << (nw & 31)) - 1u)));
    rows[rank] = c0 + nw;
    dest[e] = rank;
    mv |= rank != e;
  }
  mv = __any_sync(0xffffffffu, mv);
  if (lane == 0) moved[p] = (uint8_t)mv;
}

template <class T>
__global__ void __launch_bounds__(256) k_row_move(const MoveItem *items, int64_t nitems, const int *pair_d,
                                                  const int *pair_lb, const int *pair_ub, const int64_t *pair_roff,
                                                  const uint8_t *moved, const int *super, const int64_t *lpi,
                                                  const int64_t *lpx, const int *dest_all, T *stage_g, T *L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t it = blockIdx.x;
  if (it >= nitems) return;
  const MoveItem m = items[it];
  if (!moved[m.pair]) return;
  const int d = pair_d[m.pair], lb = pair_lb[m.pair];
  const int len = pair_ub[m.pair] - lb + 1;
  const int nrd = (int)(lpi[d + 1] - lpi[d]);
  T *Ld = L + lpx[d] + (int64_t)m.c0 * nrd + lb;
  const int *dest = dest_all + pair_roff[m.pair];
  T *vb = m.goff >= 0 ? stage_g + m.goff : reinterpret_cast<T *>(smem_raw);
  const int total = m.nc * len;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t / len, e = t - c * len;
    vb[t] = Ld[(int64_t)c * nrd + e];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t / len, e = t - c * len;
    Ld[(int64_t)c * nrd + dest[e]] = vb[t];
  }
}

// perm_new[i] = perm[c0 + locperm[i - c0]] for columns of factored supernodes.
__global__ void k_perm_compose(int n, const int *col2sup, const int *super, const uint8_t *mark,
                               const uint8_t *pivoted, const int *locperm, const int *perm, int *perm_new) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int s = col2sup[i];
    int v = perm[i];
    if ((!mark || mark[s]) && pivoted[s]) {
      int c0 = super[s];
      v = perm[c0 + locperm[i]];
    }
    perm_new[i] = v;
  }
}

__global__ void k_iperm(int n, const int *perm, int *iperm) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) iperm[perm[i]] = i;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host driver.
template <class T> static int factor_impl(Plan &P, const std::vector<int> *subset) {
  const int n = P.n;
  const int ns = P.sym.nsuper;
  cudaStream_t st = P.stream;
  T *L = reinterpret_cast<T *>(P.d_L);
  T *D = reinterpret_cast<T *>(P.d_D);
  // marks and per-level target lists
  std::vector<uint8_t> mark(ns, subset ? 0 : 1);
  if (subset)
    for (int s : *subset) {
      if (s < 0 || s >= ns) return NQG_ERR_ARG;
      mark[s] = 1;
    }
  std::vector<int> order;      // targets grouped by level
  std::vector<int> lv_small_off, lv_small_cnt, lv_glob_off, lv_glob_cnt;
  std::vector<int> row_items, lv_row_off, lv_row_cnt;  // (supernode, row block) items of k_panel_rows
  std::vector<int> tile_ids, tile_ids_tc;
  std::vector<int64_t> lv_tile_off, lv_tile_cnt, lv_tc_off, lv_tc_cnt;
  std::vector<int> map_items;  // (pair, first row) of the pair row maps, per level
  std::vector<int64_t> lv_map_off, lv_map_cnt;
  const int nlev = (int)P.levels.size();
  for (int l = 0; l < nlev; ++l) {
    int so = (int)order.size();
    for (int s : P.levels[l]) {
      const int w = P.sym.super[s + 1] - P.sym.super[s];
      if (mark[s] && w <= P.bk_small && w <= P.wide_min) order.push_back(s);
    }
    int go = (int)order.size();
    for (int s : P.levels[l]) {
      const int w = P.sym.super[s + 1] - P.sym.super[s];
      if (mark[s] && w > P.bk_small && w <= P.wide_min) order.push_back(s);
    }
    lv_small_off.push_back(so);
    lv_small_cnt.push_back(go - so);
    lv_glob_off.push_back(go);
    lv_glob_cnt.push_back((int)order.size() - go);
    lv_row_off.push_back((int)row_items.size() / 2);
    for (int q = go; q < (int)order.size(); ++q) {
      const int s = order[q];
      const int w = P.sym.super[s + 1] - P.sym.super[s];
      const int nb_rows = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]) - w;
      for (int rb = 0; rb * PR_ROWS < nb_rows; ++rb) {
        row_items.push_back(s);
        row_items.push_back(rb);
      }
    }
    lv_row_cnt.push_back((int)row_items.size() / 2 - lv_row_off.back());
    int64_t to = (int64_t)tile_ids.size();
    for (int s : P.levels[l])
      if (mark[s])
        for (int64_t t = P.tile_ptr[s]; t < P.tile_ptr[s + 1]; ++t) tile_ids.push_back((int)t);
    lv_tile_off.push_back(to);
    lv_tile_cnt.push_back((int64_t)tile_ids.size() - to);
    const int64_t tco = (int64_t)tile_ids_tc.size();
    for (int s : P.levels[l])
      if (mark[s])
        for (int64_t t = P.tile_ptr_tc[s]; t < P.tile_ptr_tc[s + 1]; ++t) tile_ids_tc.push_back((int)t);
    lv_tc_off.push_back(tco);
    lv_tc_cnt.push_back((int64_t)tile_ids_tc.size() - tco);
    const int64_t mo = (int64_t)map_items.size() / 2;
    for (int s : P.levels[l])
      if (mark[s])
        for (int q = P.pair_ptr[s]; q < P.pair_ptr[s + 1]; ++q) {
          if (P.pair_pers[q]) continue;
          const int d = P.pair_d[q];
          const int m = (int)(P.sym.lpi[d + 1] - P.sym.lpi[d]) - P.pair_lb[q];
          for (int r0 = 0; r0 < m; r0 += 256) {
            map_items.push_back(q);
            map_items.push_back(r0);
          }
        }
    lv_map_off.push_back(mo);
    lv_map_cnt.push_back((int64_t)map_items.size() / 2 - mo);
  }
  bool any = false;
  for (int s = 0; s < ns && !any; ++s) any = mark[s] != 0;
  if (!any) return NQG_OK;
  if (std::max<size_t>(order.size(), 1) > P.targets_cap) {
    if (P.d_targets) cudaFree(P.d_targets);
    P.targets_cap = std::max<size_t>(order.size(), 64);
    NQG_CUDA(cudaMalloc(&P.d_targets, P.targets_cap * sizeof(int)));
  }
  if (tile_ids.size() > P.tile_list_cap) {
    if (P.d_tile_list) cudaFree(P.d_tile_list);
    P.tile_list_cap = std::max<size_t>(tile_ids.size(), 64);
    NQG_CUDA(cudaMalloc(&P.d_tile_list, P.tile_list_cap * sizeof(int)));
  }
  // rows below the diagonal blocks of the k_bk_global supernodes: multi-CTA
  // kernel when its shared-memory staging fits, else inside k_bk_global
  int wmax_glob = 0;
  for (int q = 0; q < (int)lv_glob_off.size(); ++q)
    for (int k = lv_glob_off[q]; k < lv_glob_off[q] + lv_glob_cnt[q]; ++k)
      wmax_glob = std::max(wmax_glob, P.sym.super[order[k] + 1] - P.sym.super[order[k]]);
  const size_t pr_smem = panel_rows_smem(std::max(wmax_glob, 1), (int)sizeof(T));
  const bool rows_split = pr_smem <= 227 * 1024 && !P.panel_rows_serial;
  if (rows_split && !row_items.empty()) {
    if (row_items.size() > P.row_items_cap) {
      if (P.d_row_items) cudaFree(P.d_row_items);
      P.row_items_cap = std::max<size_t>(row_items.size(), 128);
      NQG_CUDA(cudaMalloc(&P.d_row_items, P.row_items_cap * sizeof(int)));
    }
    NQG_CUDA(cudaMemcpyAsync(P.d_row_items, row_items.data(), row_items.size() * sizeof(int), cudaMemcpyHostToDevice,
                             st));
    NQG_CUDA(cudaFuncSetAttribute(k_panel_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pr_smem));
  }
  if (!order.empty())
    NQG_CUDA(cudaMemcpyAsync(P.d_targets, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  if (!tile_ids.empty())
    NQG_CUDA(cudaMemcpyAsync(P.d_tile_list, tile_ids.data(), tile_ids.size() * sizeof(int), cudaMemcpyHostToDevice,
                             st));
  if (tile_ids_tc.size() > P.tile_list_tc_cap) {
    if (P.d_tile_list_tc) cudaFree(P.d_tile_list_tc);
    P.tile_list_tc_cap = std::max<size_t>(tile_ids_tc.size(), 64);
    NQG_CUDA(cudaMalloc(&P.d_tile_list_tc, P.tile_list_tc_cap * sizeof(int)));
  }
  if (!tile_ids_tc.empty())
    NQG_CUDA(cudaMemcpyAsync(P.d_tile_list_tc, tile_ids_tc.data(), tile_ids_tc.size() * sizeof(int),
                             cudaMemcpyHostToDevice, st));
  if (!tile_ids_tc.empty())
    NQG_CUDA(cudaFuncSetAttribute(k_update_t5, cudaFuncAttributeMaxDynamicSharedMemorySize, t5::smem_bytes(1)));
  if (map_items.size() > P.map_items_cap) {
    if (P.d_map_items) cudaFree(P.d_map_items);
    P.map_items_cap = std::max<size_t>(map_items.size(), 128);
    NQG_CUDA(cudaMalloc(&P.d_map_items, P.map_items_cap * sizeof(int)));
  }
  if (!map_items.empty())
    NQG_CUDA(cudaMemcpyAsync(P.d_map_items, map_items.data(), map_items.size() * sizeof(int), cudaMemcpyHostToDevice,
                             st));
  uint8_t *d_mark = P.d_pivoted + ns;  // second half of the pivoted buffer holds the marks
  NQG_CUDA(cudaMemcpyAsync(d_mark, mark.data(), ns, cudaMemcpyHostToDevice, st));
  NQG_CUDA(cudaMemsetAsync(P.d_pivoted, 0, ns, st));
  // reset + assemble
  if (!subset) {
    NQG_CUDA(cudaMemsetAsync(L, 0, (size_t)P.sym.xsize * sizeof(T), st));
    NQG_CUDA(cudaMemsetAsync(D, 0, (size_t)2 * n * sizeof(T), st));
  } else {
    // every supernode being refactored, staged in the permutation scratch
    // buffer (n >= nsuper ints; its later users run after this kernel)
    std::vector<int> all_marked;
    for (int s = 0; s < ns; ++s)
      if (mark[s]) all_marked.push_back(s);
    NQG_CUDA(cudaMemcpyAsync(P.d_perm_tmp, all_marked.data(), all_marked.size() * sizeof(int),
                             cudaMemcpyHostToDevice, st));
    k_zero_targets<T><<<(unsigned)all_marked.size(), 256, 0, st>>>(P.d_perm_tmp, (int)all_marked.size(), P.d_super,
                                                                   P.d_lpi, P.d_lpx, L, D, n);
    P.nlaunch++;
  }
  {
    int blocks = std::min(std::max((n + 7) / 8, 1), 4096);
    cudaEvent_t e0 = P.prof_begin();
    k_assemble<T><<<blocks, 256, 0, st>>>(n, P.d_Kp, P.d_Ki, P.d_Kx, P.d_iperm, P.d_col2sup, P.d_super, P.d_lpi,
                                          P.d_lpx, P.d_ls, subset ? d_mark : nullptr, L, P.d_status);
    P.prof_end(NQG_K_OTHER, e0, 0.0, 0.0);
    P.nlaunch++;
  }
  const size_t smem_small = (size_t)(BK_SMALL * BK_SMALL + BK_SMALL * BK_THREADS) * sizeof(T);
  static bool attr_set[2] = {false, false};
  int ai = sizeof(T) == 8 ? 0 : 1;
  if (!attr_set[ai]) {
    NQG_CUDA(cudaFuncSetAttribute(k_bk_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_small));
    attr_set[ai] = true;
  }
  auto bk_flops = [&](int s) {
    const double w = P.sym.super[s + 1] - P.sym.super[s], r = (double)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
    // sum_{k<w} (r-k)^2, the conventional factorization flop count of one supernode
    return w * r * r - r * w * (w - 1) + (w - 1) * w * (2 * w - 1) / 6.0;
  };
  for (int l = 0; l < nlev; ++l) {
    if (lv_tile_cnt[l] + lv_tc_cnt[l] > 0) {
      double fl = 0;
      if (P.prof)
        for (int s : P.levels[l])
          if (mark[s])
            for (int q = P.pair_ptr[s]; q < P.pair_ptr[s + 1]; ++q)
              if (!P.pair_pers[q]) fl += P.pair_flops[q];
      cudaEvent_t e0 = P.prof_begin();
      if (lv_map_cnt[l] > 0) {
        k_pair_rowmap<<<(unsigned)lv_map_cnt[l], 256, 0, st>>>(
            reinterpret_cast<const int2 *>(P.d_map_items) + lv_map_off[l], P.d_pair_s, P.d_pair_d, P.d_pair_lb,
            P.d_pair_moff, P.d_super, P.d_lpi, P.d_ls, P.d_pair_map, P.d_status);
        P.nlaunch++;
      }
      if (lv_tile_cnt[l] > 0) {
        k_update<T><<<(unsigned)lv_tile_cnt[l], UPD_THREADS, 0, st>>>(P.d_tiles, P.d_tile_list + lv_tile_off[l],
                                                                      (int)lv_tile_cnt[l], n, P.d_super, P.d_lpi,
                                                                      P.d_lpx, P.d_ls, L, D, P.d_status,
                                                                      P.d_pair_map, P.d_pair_moff, P.d_pair_lb);
        P.nlaunch++;
      }
      if constexpr (sizeof(T) == 4) {
        if (lv_tc_cnt[l] > 0) {
          k_update_t5<<<(unsigned)lv_tc_cnt[l], t5::THREADS, t5::smem_bytes(1), st>>>(
              P.d_tiles_tc, P.d_tile_list_tc + lv_tc_off[l], n, P.d_super, P.d_lpi, P.d_lpx, P.d_ls, L, D,
              P.d_status, P.d_pair_map, P.d_pair_moff, P.d_pair_lb);
          P.nlaunch++;
        }
      }
      P.prof_end(NQG_K_UPDATE, e0, fl, 0.0);
    }
    if constexpr (sizeof(T) == 4) {
      // the largest pairs of this level, one persistent launch each
      for (int s : P.levels[l])
        if (mark[s])
          for (int k = P.pers_ptr[s]; k < P.pers_ptr[s + 1]; ++k) {
            int rc = update_pair_persistent(P, s, P.pers_pair[k], L, D);
            if (rc) return rc;
          }
    }
    if (lv_small_cnt[l] + lv_glob_cnt[l] > 0) {
      double fl = 0;
      if (P.prof)
        for (int q = lv_small_off[l]; q < lv_glob_off[l] + lv_glob_cnt[l]; ++q) fl += bk_flops(order[q]);
      cudaEvent_t e0 = P.prof_begin();
      if (lv_small_cnt[l] > 0) {
        k_bk_small<T><<<lv_small_cnt[l], BK_THREADS, smem_small, st>>>(P.d_targets + lv_small_off[l], n, P.d_super,
                                                                        P.d_lpi, P.d_lpx, L, D, P.d_locperm,
                                                                        P.d_pivoted, P.d_status);
        P.nlaunch++;
      }
      if (lv_glob_cnt[l] > 0) {
        // diagonal blocks staged in shared memory when the widest fits
        int wl = 0;
        for (int q = lv_glob_off[l]; q < lv_glob_off[l] + lv_glob_cnt[l]; ++q)
          wl = std::max(wl, P.sym.super[order[q] + 1] - P.sym.super[order[q]]);
        const size_t bks = (size_t)wl * wl * sizeof(T);
        const int staged = bks <= BKG_STAGE_MAX ? 1 : 0;
        if (staged)
          NQG_CUDA(cudaFuncSetAttribute(k_bk_global<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)BKG_STAGE_MAX));
        k_bk_global<T><<<lv_glob_cnt[l], 256, staged ? bks : 0, st>>>(
            P.d_targets + lv_glob_off[l], n, P.d_super, P.d_lpi, P.d_lpx, L, D, P.d_locperm, P.d_pivoted,
            P.d_perm_tmp, rows_split ? 0 : 1, P.d_status, staged);
        P.nlaunch++;
        if (rows_split && lv_row_cnt[l] > 0) {
          k_panel_rows<T><<<lv_row_cnt[l], 256, pr_smem, st>>>(
              reinterpret_cast<const int2 *>(P.d_row_items) + lv_row_off[l], n, P.d_super, P.d_lpi, P.d_lpx, L, D,
              P.d_locperm, P.d_pivoted);
          P.nlaunch++;
        }
      }
      P.prof_end(NQG_K_BK, e0, fl, 0.0);
    }
    for (int s : P.levels[l]) {
      if (!mark[s] || P.sym.super[s + 1] - P.sym.super[s] <= P.wide_min) continue;
      int rc = factor_wide<T>(P, s, L, D, P.wide_nb, reinterpret_cast<T *>(P.d_wide_W),
                              reinterpret_cast<WideCtl *>(P.d_wide_ctl), P.num_sms);
      if (rc) return rc;
    }
  }
  NQG_CUDA(cudaGetLastError());
  // row renaming in descendants of pivoted supernodes
  {
    const int64_t npairs = (int64_t)P.pair_d.size();
    if (npairs > 0) {
      cudaEvent_t e0 = P.prof_begin();
      const int blocks_n = std::min((n + 255) / 256, 4096);
      k_loc_inverse<<<blocks_n, 256, 0, st>>>(n, P.d_col2sup, P.d_super, P.d_pivoted, P.d_locperm, P.d_locinv);
      const size_t warp_bytes = (size_t)2 * P.rr_words * sizeof(unsigned);
      int wpb = (int)std::min<size_t>(8, std::max<size_t>(1, (48 * 1024) / warp_bytes));
      const size_t rn_smem = warp_bytes * wpb;
      if (rn_smem > 227 * 1024) return NQG_ERR_SIZE;
      static size_t rn_set = 0;
      if (rn_smem > 48 * 1024 && rn_smem > rn_set) {
        NQG_CUDA(cudaFuncSetAttribute(k_row_rename, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rn_smem));
        rn_set = rn_smem;
      }
      const int64_t rn_blocks = (npairs + wpb - 1) / wpb;
      k_row_rename<<<(unsigned)rn_blocks, 32 * wpb, rn_smem, st>>>(
          P.d_pair_s, P.d_pair_d, P.d_pair_lb, P.d_pair_ub, npairs, P.d_pair_roff, P.d_pivoted, P.d_super, P.d_lpi,
          P.d_ls, P.d_locinv, P.d_rr_dest, P.d_rr_moved, P.rr_words, P.d_status);
      P.nlaunch += 2;
      T *stage = reinterpret_cast<T *>(P.d_rr_stage);
      if (P.rr_items_small > 0) {
        k_row_move<T><<<(unsigned)P.rr_items_small, 256, RR_STAGE_BYTES, st>>>(
            P.d_rr_items, P.rr_items_small, P.d_pair_d, P.d_pair_lb, P.d_pair_ub, P.d_pair_roff, P.d_rr_moved,
            P.d_super, P.d_lpi, P.d_lpx, P.d_rr_dest, stage, L);
        P.nlaunch++;
      }
      if (P.rr_items_big > 0) {
        static size_t mv_set[2] = {0, 0};
        const size_t big = std::max<size_t>(P.rr_big_smem, 16);
        if (big > 48 * 1024 && big > mv_set[ai]) {
          NQG_CUDA(cudaFuncSetAttribute(k_row_move<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)big));
          mv_set[ai] = big;
        }
        k_row_move<T><<<(unsigned)P.rr_items_big, 256, big, st>>>(
            P.d_rr_items + P.rr_items_small, P.rr_items_big, P.d_pair_d, P.d_pair_lb, P.d_pair_ub, P.d_pair_roff,
            P.d_rr_moved, P.d_super, P.d_lpi, P.d_lpx, P.d_rr_dest, stage, L);
        P.nlaunch++;
      }
      P.prof_end(NQG_K_OTHER, e0, 0.0, 0.0);
    }
  }
  {
    int blocks = std::min((n + 255) / 256, 4096);
    k_perm_compose<<<blocks, 256, 0, st>>>(n, P.d_col2sup, P.d_super, d_mark, P.d_pivoted, P.d_locperm, P.d_perm,
                                           P.d_perm_tmp);
    std::swap(P.d_perm, P.d_perm_tmp);
    k_iperm<<<blocks, 256, 0, st>>>(n, P.d_perm, P.d_iperm);
    P.nlaunch += 2;
  }
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

int dev_factor(Plan &P, const std::vector<int> *subset) {
  P.tinv_valid = false;  // the block solves form their tile inverses again
  if (P.set.precision == NQG_FP32) return factor_impl<float>(P, subset);
  return factor_impl<double>(P, subset);
}

}  // namespace nqg
