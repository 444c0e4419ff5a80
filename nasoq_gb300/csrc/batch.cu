// Batched NASOQ: thousands of small QPs of uneven size, each solved to the
// end by one CTA of a persistent kernel -- the dual active-set iteration
// (reference Nasoq::numeric_QP, src/nasoq.cpp:478-610), its SoMod partial
// refactorizations (update_ldl_left_sn_02_v2, src/ldl/Serial_update_ldl.cpp:
// 18-277), masked supernodal solves and GMRES refinement all run on the
// device; the host only fills the work queue.
//
// Per problem, in the CTA's scratch slot (or, for the factor and its row
// lists, in shared memory when they fit the launch's staging space):
//  * the supernodal factor in the reference's BCSC layout (column-major
//    nrow x w blocks, D as diagonal + 2x2 sub-diagonal halves), the composed
//    ordering perm/iperm and the row lists, renamed after Bunch-Kaufman
//    pivoting as the reference's row_reordering does (without re-sorting the
//    renamed rows: every consumer maps them through the target's row list).
//    Once a supernode is factored, the unit lower triangle of its diagonal
//    block is replaced by its inverse, which is all the solves need of it;
//  * the active set as a per-constraint flag.  Hidden (inactive) constraint
//    columns are width-1 supernodes whose entries read as zero; the
//    reference's hidden-column tree edits (linear_solver_wrapper.cpp:770-907)
//    become a visibility flag per supernode plus, per supernode, a bit mask
//    of its active constraint-column descendants, and the supernodes to
//    refactor after an edit are those on the elimination-tree paths from the
//    edited column and its variables to the root;
//  * two copies of K's values in CSR order (factorization values with the
//    regularization, refinement values without it), edited in place;
//  * the KKT vectors in the original numbering; the triangular solves gather
//    them into shared memory in the factor's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "batch.hpp"
#include "bk.cuh"

namespace nqg {

namespace {

// Up to 256 threads per CTA; the kernel's natural 128 registers leave 4 CTAs
// of 128 threads per SM.  (Capping it at 80 registers for 6 CTAs per SM was
// measured slower: 7-12 % on cold and FP64 batches, +2 % on warm ones.)
constexpr int BT_MAX_THREADS = 256;
constexpr int WF_WARPS = 4;  // warps of the level-parallel factorization
constexpr int MR_CAP = BATCH_MR_CAP;  // Krylov steps per restart held in shared memory

template <class T> struct Ctx {
  // pattern (read-only)
  int n, meq, mineq, N, base, ns, nlev, nnzR, cmask_ok;
  const int *__restrict__ super, *__restrict__ sparent, *__restrict__ col2sup, *__restrict__ lpi, *__restrict__ lpx;
  const int *__restrict__ lvl_ptr, *__restrict__ lvl_sn, *__restrict__ lev;
  const int *__restrict__ Rp, *__restrict__ Rj, *__restrict__ Rq, *__restrict__ ent;
  const int *__restrict__ bt_ptr, *__restrict__ bt_var, *__restrict__ bt_q, *__restrict__ bt_rpos;
  const int *__restrict__ sn_con, *__restrict__ con_sn, *__restrict__ eq_ptr, *__restrict__ eq_var,
      *__restrict__ eq_q;
  const int4 *__restrict__ snrec;  // 2 per supernode: {c0, w, nrow, value offset}, {row-list offset, pairs}
  const int4 *__restrict__ prec;   // per pair: {descendant, lb, ub, descendant's row-list offset}
  const int *__restrict__ con_ptr, *__restrict__ con_tgt;
  const uint8_t *__restrict__ sn_big;  // per supernode: solved by a warp (wide or tall block)
  // problem
  const double *__restrict__ kv, *__restrict__ q, *__restrict__ bq, *__restrict__ dq;
  const uint8_t *__restrict__ pert;
  double reg, reg32;
  // slot
  T *L, *D;
  int *ls, *perm, *iperm, *lperm, *alist, *vlist, *mlist;
  uint8_t *mark, *piv;
  double *Fv, *Rv;  // factorization / refinement values of K in CSR order
  unsigned long long *cmask;  // per supernode: active constraint-column descendants (bit = pair - pair_mid)
  double *rhs, *sol, *r, *w, *V, *tmp;
  T *Z;
  // shared memory
  int *map;
  T *xs, *B, *rowbuf, *Dsm, *Esm, *Binv;
  int *lp;
  // per-warp scratch of the level-parallel factorization (WF_WARPS warps):
  // block wcap x rcap, D, E, local pivot order, Bunch-Kaufman multipliers
  T *wB, *wD, *wE, *wwk;
  int *wlp;
  int wcap, rcap;  // widest / tallest supernode a warp takes (<= 32)
  int wf;          // level-parallel factorization on
  uint8_t *vis;  // per supernode: visible (structural, or the column of an active constraint)
  uint8_t *act;  // per constraint: active
  int *vlvl;     // visible supernodes of each level: vlist[vlvl[l] .. vlvl[l+1]),
  int *vmid;     // the small ones (a thread each) before vmid[l], the big ones (a warp each) after
  int *vfill;    // 2 * (nlev + 1) fill counters of build_vlist
  int *nmark;    // length of mlist
  double *red;   // 32 doubles
  int *redi;     // 32 ints
  int *status;   // device status bits of this problem
  unsigned long long *cyc;  // per-phase SM cycles of this CTA (profiling), or null
};

// Counters of nqg_batch_get_profile.
enum { PH_TOTAL, PH_INIT, PH_FACTOR, PH_PRECOND, PH_SPMV, PH_REFINE, PH_SELECT, PH_UPDATE, PH_SN, PH_ITER,
       PH_FWD_WIDE, PH_FWD_NARROW, PH_DIAG, PH_BWD, PH_GATHER, PH_INIT_FACTOR,
       PH_SN_ASSEMBLE, PH_SN_UPDATES, PH_SN_BK, PH_SN_ROWS, PH_SN_INVERSE, PH_SN_STORE, PH_RENAME, PH_N };
static_assert(PH_N <= BATCH_PROFILE_COUNTERS, "profile counters");
#define BQ_T0(c) const long long t0_ = (c).cyc ? clock64() : 0
#define BQ_T1(c, ph) \
  if ((c).cyc && threadIdx.x == 0) (c).cyc[ph] += (unsigned long long)(clock64() - t0_)

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }
__device__ __forceinline__ int num_warps() { return blockDim.x >> 5; }

template <class T> __device__ __forceinline__ bool visible(const Ctx<T> &c, int s) { return c.vis[s] != 0; }

// Calls f(pair) for every descendant pair of s whose descendant is visible:
// the structural ones, then the active constraint columns (bit mask, or a
// scan when a supernode has more than 64 of them).
template <class T, class F> __device__ __forceinline__ void for_visible_pairs(const Ctx<T> &c, int s, int pp, int pm,
                                                                              int pe, F &&f) {
  for (int pq = pp; pq < pm; ++pq) f(pq);
  if (c.cmask_ok) {
    unsigned long long m = c.cmask[s];
    while (m) {
      const int b = __ffsll((long long)m) - 1;
      m &= m - 1ull;
      f(pm + b);
    }
  } else {
    for (int pq = pm; pq < pe; ++pq)
      if (c.vis[c.prec[pq].x]) f(pq);
  }
}

// Block-wide sum in a fixed order (per-thread strided partials, then a tree):
// the same inputs give the same bits on every run.
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane_id() == 0) red[warp_id()] = v;
  __syncthreads();
  if (warp_id() == 0) {
    v = lane_id() < num_warps() ? red[lane_id()] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0) red[0] = v;
  }
  __syncthreads();
  v = red[0];
  __syncthreads();
  return v;
}

__device__ int block_sum_int(int v, int *redi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane_id() == 0) redi[warp_id()] = v;
  __syncthreads();
  if (warp_id() == 0) {
    v = lane_id() < num_warps() ? redi[lane_id()] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0) redi[0] = v;
  }
  __syncthreads();
  v = redi[0];
  __syncthreads();
  return v;
}

// Block-wide selection: the largest (sel_max) or smallest value, the
// smallest index winning ties -- the outcome of the reference's ascending
// scans with strict comparisons.  idx < 0 marks "no candidate".
__device__ void block_select(double &v, int &idx, bool sel_max, double *red, int *redi) {
  auto better = [&](double ov, int oi, double cv, int ci) {
    if (oi < 0) return false;
    if (ci < 0) return true;
    if (ov == cv) return oi < ci;
    return sel_max ? ov > cv : ov < cv;
  };
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, v, o);
    int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (better(ov, oi, v, idx)) {
      v = ov;
      idx = oi;
    }
  }
  __syncthreads();
  if (lane_id() == 0) {
    red[warp_id()] = v;
    redi[warp_id()] = idx;
  }
  __syncthreads();
  if (warp_id() == 0) {
    v = lane_id() < num_warps() ? red[lane_id()] : 0.0;
    idx = lane_id() < num_warps() ? redi[lane_id()] : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, v, o);
      int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (better(ov, oi, v, idx)) {
        v = ov;
        idx = oi;
      }
    }
    if (lane_id() == 0) {
      red[0] = v;
      redi[0] = idx;
    }
  }
  __syncthreads();
  v = red[0];
  idx = redi[0];
  __syncthreads();
}


// ---- values ---------------------------------------------------------------
// Factorization value of lower-CSC entry vq: inactive constraint entries read
// as zero (the reference zeroes them in its ordered matrix), perturbed
// diagonals as the regularization (find_perturbation,
// linear_solver_wrapper.cpp:352-363).
//
// An FP32 factor also gets a sign-keeping floor reg32 on its diagonal: pivots
// as small as the 1e-9 regularization create element growth of ~1e9 under
// Bunch-Kaufman restricted to supernode diagonal blocks, beyond what FP32
// carries; the factor is only the preconditioner of the FP64 refinement,
// whose matrix keeps the reference's values.
template <class T> __device__ __forceinline__ double fact_val(const Ctx<T> &c, int vq) {
  const int e = c.ent[vq];
  double v = c.kv[vq];
  if (e >= 0) return c.act[e] ? v : 0.0;
  if (e <= -2) {
    if (c.pert[-2 - e]) v = c.reg;
    if (sizeof(T) == 4 && fabs(v) < c.reg32) v = v < 0.0 ? -c.reg32 : c.reg32;
  }
  return v;
}
// Refinement value: perturbed diagonals read as zero (set_diags(0),
// linear_solver_wrapper.cpp:1359-1394).
template <class T> __device__ __forceinline__ double ref_val(const Ctx<T> &c, int vq) {
  const int e = c.ent[vq];
  double v = c.kv[vq];
  if (e >= 0) return c.act[e] ? v : 0.0;
  if (e <= -2 && c.pert[-2 - e]) return 0.0;
  return v;
}

// Panel rows [w, nr) of the supernode block B (ld nr): columns permuted by
// the pivot order, solved with the unit lower L11^T, scaled by D^-1 (1x1:
// times 1/d; 2x2: Cramer's rule, the arithmetic of blocked_2by2_solver,
// Sym_BLAS.cpp:492-529).  Warp 0, one lane per row, rows staged in rowbuf
// (w x 32).
template <class T> __device__ void panel_rows_warp0(Ctx<T> &c, T *B, int nr, int w, bool permute) {
  if (warp_id() != 0) return;
  const int lane = lane_id();
  T *rb = c.rowbuf;
  const T *D = c.Dsm, *E = c.Esm;
  for (int r0 = w; r0 < nr; r0 += 32) {
    const int r = r0 + lane;
    if (r < nr) {
      for (int j = 0; j < w; ++j) rb[j * 32 + lane] = B[r + (size_t)(permute ? c.lp[j] : j) * nr];
      for (int j = 0; j < w; ++j) {
        T x = rb[j * 32 + lane];
        for (int t = 0; t < j; ++t) x -= rb[t * 32 + lane] * B[j + (size_t)t * nr];
        rb[j * 32 + lane] = x;
      }
      for (int j = 0; j < w; ++j) {
        if (E[j] == T(0) || j + 1 >= w) {
          B[r + (size_t)j * nr] = rb[j * 32 + lane] * (T(1) / D[j]);
        } else {
          const T e = E[j];
          const T inv = T(1) / (D[j] * D[j + 1] - e * e);
          const T x1 = rb[j * 32 + lane], x2 = rb[(j + 1) * 32 + lane];
          B[r + (size_t)j * nr] = (x1 * D[j + 1] - x2 * e) * inv;
          B[r + (size_t)(j + 1) * nr] = (x2 * D[j] - x1 * e) * inv;
          ++j;
        }
      }
    }
  }
  __syncwarp();
}

// Subtracts descendant d's L D L^T restricted to target s (rows lb.. of d,
// columns lb..ub) from the staged target block B.  One warp per pair; pairs
// of different warps may hit the same entries, so the subtraction is atomic
// (the summation order of a target entry varies between runs, as in the
// reference's threaded factorization).
template <class T> __device__ void sub_update_warp(Ctx<T> &c, int pq, int d, int c0, int w, int nr, const int *rows) {
  const int lane = lane_id();
  const int4 pr = c.prec[pq], d0 = c.snrec[2 * d];
  const int lb = pr.y, ub = pr.z;
  const int cd = d0.x, wd = d0.y, nrd = d0.z;
  const int *rd = c.ls + pr.w;
  const T *Ld = c.L + d0.w;
  const T *Dd = c.D + cd, *Ed = c.D + c.N + cd;
  const int m = nrd - lb, nc = ub - lb + 1;
  T *B = c.B;
  // lanes over the descendant's rows (each lane's target row found once),
  // the target columns in turn; the products accumulate in the factor's
  // precision, in the order of the descendant's columns
  for (int i0 = 0; i0 < m; i0 += 32) {
    const int i = i0 + lane;
    int ti = -1;
    if (i < m) {
      const int ri = rd[lb + i];
      ti = c.map[ri];
      if (ti < 0 || ti >= nr || rows[ti] != ri) {
        atomicOr(c.status, ST_BOUNDS);
        ti = -1;
      }
    }
    for (int jj = 0; jj < nc; ++jj) {
      const int tj = rd[lb + jj] - c0;
      if (tj < 0 || tj >= w) {
        if (lane == 0) atomicOr(c.status, ST_BOUNDS);
        continue;
      }
      if (ti < tj) continue;  // lower triangle of the target only (and rows out of bounds)
      T acc = T(0);
      for (int k = 0; k < wd; ++k) {
        const T lik = Ld[lb + i + (size_t)k * nrd];
        const T ek = Ed[k];
        if (ek == T(0) || k + 1 >= wd) {
          acc += lik * Dd[k] * Ld[lb + jj + (size_t)k * nrd];
        } else {
          // 2x2 block (k, k+1): (D L^T)_k,j = d1 L_jk + e L_j,k+1; (D L^T)_k+1,j = e L_jk + d2 L_j,k+1
          const T ljk = Ld[lb + jj + (size_t)k * nrd], ljk1 = Ld[lb + jj + (size_t)(k + 1) * nrd];
          const T lik1 = Ld[lb + i + (size_t)(k + 1) * nrd];
          acc += lik * (Dd[k] * ljk + ek * ljk1) + lik1 * (ek * ljk + Dd[k + 1] * ljk1);
          ++k;
        }
      }
      atomicAdd(&B[ti + tj * nr], -acc);
    }
  }
}

// Warp-wide argmax of |value| with the smallest index winning ties (the
// LAPACK idamax convention); every lane returns the winner.
template <class T> __device__ __forceinline__ void warp_argmax(T &v, int &idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (oi >= 0 && (idx < 0 || ov > v || (ov == v && oi < idx))) {
      v = ov;
      idx = oi;
    }
  }
}

template <class T> __device__ __forceinline__ void s_flag_store(Ctx<T> &c, bool f) { c.redi[31] = f ? 1 : 0; }

// Bunch-Kaufman (alpha = (1+sqrt(17))/8, the LAPACK dsytf2('L') pivot rule
// and the reference's reorder_after_sytrf form: explicit interchanges, L with
// unit diagonal, D / E the diagonal and 2x2 sub-diagonals, perm[m] = original
// local column at position m) on a w <= 32 wide lower-stored block, by one
// warp: the steps and the arithmetic of each entry are those of the CTA-wide
// bk_factor.  wk holds the multipliers of a step (w - 1 of a 1x1, 2 (w - 2) of a
// 2x2).  Returns whether
// any interchange happened.
template <class T>
__device__ bool bk_factor_warp(T *a, int lda, int w, T *D, T *E, int *perm, int *status, T *wk) {
  const T alpha = (T)((1.0 + sqrt(17.0)) / 8.0);
  const int lane = lane_id();
  bool pivoted = false;
  for (int m = lane; m < w; m += 32) perm[m] = m;
  __syncwarp();
  int k = 0;
  while (k < w) {
    const T absakk = tabs(a[k + (size_t)k * lda]);
    T cv = T(-1);
    int ci = -1;
    for (int i = k + 1 + lane; i < w; i += 32) {
      const T v = tabs(a[i + (size_t)k * lda]);
      if (ci < 0 || v > cv) {
        cv = v;
        ci = i;
      }
    }
    warp_argmax(cv, ci);
    const T colmax = ci >= 0 ? cv : T(0);
    const int imax = ci;
    int kp = k, kstep = 1, zero = 0;
    if ((absakk >= colmax ? absakk : colmax) == T(0) || absakk != absakk) {
      zero = 1;
    } else if (absakk >= alpha * colmax) {
      kp = k;
    } else {
      T rv = T(-1);
      int ri = -1;
      for (int j = k + lane; j < w; j += 32) {
        if (j == imax) continue;
        const T v = j < imax ? tabs(a[imax + (size_t)j * lda]) : tabs(a[j + (size_t)imax * lda]);
        if (ri < 0 || v > rv) {
          rv = v;
          ri = j;
        }
      }
      warp_argmax(rv, ri);
      const T rowmax = rv;
      if (absakk >= alpha * colmax * (colmax / rowmax)) {
        kp = k;
      } else if (tabs(a[imax + (size_t)imax * lda]) >= alpha * rowmax) {
        kp = imax;
      } else {
        kp = imax;
        kstep = 2;
      }
    }
    const int kk = k + kstep - 1;
    if (zero && lane == 0) atomicOr(status, absakk == absakk ? ST_ZERO_PIVOT : ST_NONFINITE);
    if (kp != kk) {  // symmetric interchange of kk and kp (kp > kk)
      pivoted = true;
      for (int i = kp + 1 + lane; i < w; i += 32) {
        const T t = a[i + (size_t)kk * lda];
        a[i + (size_t)kk * lda] = a[i + (size_t)kp * lda];
        a[i + (size_t)kp * lda] = t;
      }
      for (int j = kk + 1 + lane; j < kp; j += 32) {
        const T t = a[j + (size_t)kk * lda];
        a[j + (size_t)kk * lda] = a[kp + (size_t)j * lda];
        a[kp + (size_t)j * lda] = t;
      }
      const int ncols_left = kstep == 2 ? k + 1 : k;
      for (int cc = lane; cc < ncols_left; cc += 32) {
        const T t = a[kk + (size_t)cc * lda];
        a[kk + (size_t)cc * lda] = a[kp + (size_t)cc * lda];
        a[kp + (size_t)cc * lda] = t;
      }
      if (lane == 0) {
        const T t = a[kk + (size_t)kk * lda];
        a[kk + (size_t)kk * lda] = a[kp + (size_t)kp * lda];
        a[kp + (size_t)kp * lda] = t;
        const int pt = perm[kk];
        perm[kk] = perm[kp];
        perm[kp] = pt;
      }
    }
    __syncwarp();
    if (kstep == 1) {
      if (!zero) {
        const T r1 = T(1) / a[k + (size_t)k * lda];
        // trailing update of the lower triangle: lane owns row i = k + 1 + lane
        // (w <= 32) and walks its columns j <= i, independent updates; the
        // multipliers r1 a_jk are staged once per column
        for (int j = k + 1 + lane; j < w; j += 32) wk[j] = r1 * a[j + (size_t)k * lda];
        __syncwarp();
        {
          const int i = k + 1 + lane;
          if (i < w) {
            const T aik = a[i + (size_t)k * lda];
            for (int j = k + 1; j <= i; ++j) a[i + (size_t)j * lda] -= wk[j] * aik;
          }
        }
        __syncwarp();
        for (int i = k + 1 + lane; i < w; i += 32) a[i + (size_t)k * lda] *= r1;
      }
      if (lane == 0) {
        D[k] = a[k + (size_t)k * lda];
        E[k] = T(0);
      }
    } else {
      // 2x2 pivot on rows/cols k, k+1
      T d21 = a[k + 1 + (size_t)k * lda];
      const T d11 = a[k + 1 + (size_t)(k + 1) * lda] / d21;
      const T d22 = a[k + (size_t)k * lda] / d21;
      const T t = T(1) / (d11 * d22 - T(1));
      d21 = t / d21;
      const int m = w - k - 2;
      for (int q = lane; q < m; q += 32) {
        const int j = k + 2 + q;
        const T ajk = a[j + (size_t)k * lda], ajk1 = a[j + (size_t)(k + 1) * lda];
        wk[2 * q] = d21 * (d11 * ajk - ajk1);
        wk[2 * q + 1] = d21 * (d22 * ajk1 - ajk);
      }
      __syncwarp();
      {
        // lane owns row i = k + 2 + lane (w <= 32), independent updates over its columns
        const int i = k + 2 + lane;
        if (i < w) {
          const T aik = a[i + (size_t)k * lda], aik1 = a[i + (size_t)(k + 1) * lda];
          for (int q = 0; q <= i - k - 2; ++q)
            a[i + (size_t)(k + 2 + q) * lda] -= aik * wk[2 * q] + aik1 * wk[2 * q + 1];
        }
      }
      __syncwarp();
      for (int q = lane; q < m; q += 32) {
        const int j = k + 2 + q;
        a[j + (size_t)k * lda] = wk[2 * q];
        a[j + (size_t)(k + 1) * lda] = wk[2 * q + 1];
      }
      __syncwarp();
      if (lane == 0) {
        D[k] = a[k + (size_t)k * lda];
        D[k + 1] = a[k + 1 + (size_t)(k + 1) * lda];
        E[k] = a[k + 1 + (size_t)k * lda];
        E[k + 1] = T(0);
        a[k + 1 + (size_t)k * lda] = T(0);
      }
    }
    __syncwarp();
    k += kstep;
  }
  for (int m = lane; m < w; m += 32) a[m + (size_t)m * lda] = T(1);
  __syncwarp();
  return pivoted;
}

// ---- factorization of one supernode (CTA scope) ------------------------------
// Left-looking step of the reference (Serial_update_ldl.cpp:62-190): scatter
// the matrix columns, subtract every visible descendant's L D L^T restricted
// to the supernode, Bunch-Kaufman on the diagonal block, permute / solve /
// scale the rows below.
template <class T> __device__ void factor_sn(Ctx<T> &c, int s) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (c.cyc && tid == 0) c.cyc[PH_SN] += 1;
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const int *rows = c.ls + r1.x;
  T *B = c.B;
  long long tq = c.cyc ? clock64() : 0;
  auto lap = [&](int ph) {
    if (c.cyc && tid == 0) {
      const long long now = clock64();
      c.cyc[ph] += (unsigned long long)(now - tq);
      tq = now;
    }
  };
  for (int p = tid; p < nr; p += nt) c.map[rows[p]] = p;
  for (int e = tid; e < nr * w; e += nt) B[e] = T(0);
  __syncthreads();
  // matrix columns (symmetric neighbours of the original column, ordered >=
  // the column): g threads per column, all columns at once
  const int g = w < nt ? nt / w : 1;
  for (int t = tid; t < w * g; t += nt) {
    const int m = t % w, k0 = t / w;
    const int col = c0 + m;
    const int j = c.perm[col];
    for (int qq = c.Rp[j] + k0; qq < c.Rp[j + 1]; qq += g) {
      const int oi = c.iperm[c.Rj[qq]];
      if (oi < col) continue;
      const int pos = c.map[oi];
      if (pos < 0 || pos >= nr || rows[pos] != oi) {  // not in the row list: corrupted structure
        atomicOr(c.status, ST_BOUNDS);
        continue;
      }
      B[pos + m * nr] = T(c.Fv[qq]);
    }
  }
  __syncthreads();
  lap(PH_SN_ASSEMBLE);
  // descendant updates: descendants that never hide, then the active
  // constraint columns; warp wi takes every num_warps()-th of them
  {
    int t = 0;
    const int wi = warp_id(), nw = num_warps();
    for_visible_pairs(c, s, r1.y, r1.z, r1.w, [&](int pq) {
      if (t++ % nw == wi) sub_update_warp(c, pq, c.prec[pq].x, c0, w, nr, rows);
    });
  }
  __syncthreads();
  lap(PH_SN_UPDATES);
  // Bunch-Kaufman on the diagonal block (one warp up to 32 columns), then the rows below
  bool pivoted = false;
  if (w <= 32) {
    if (warp_id() == 0) {
      const bool pv = bk_factor_warp<T>(B, nr, w, c.Dsm, c.Esm, c.lp, c.status, c.rowbuf);
      if (lane_id() == 0) s_flag_store(c, pv);
    }
    __syncthreads();
    pivoted = c.redi[31] != 0;
    __syncthreads();
  } else {
    bk_factor<T>(B, nr, w, c.Dsm, c.Esm, c.lp, c.status, &pivoted);
  }
  __syncthreads();
  lap(PH_SN_BK);
  if (nr > w) panel_rows_warp0(c, B, nr, w, pivoted);
  __syncthreads();
  lap(PH_SN_ROWS);
  // The solves apply the diagonal block through the inverse of its unit
  // lower triangle (one product instead of w dependent steps); nothing else
  // reads L11 once the rows below are solved, so the inverse replaces it.
  // Column j of the inverse by thread j: X[i][j] = -sum_{j<=k<i} L[i][k] X[k][j].
  for (int j = tid; j < w; j += nt) {
    T *X = c.Binv;
    X[j + j * w] = T(1);
    for (int i = j + 1; i < w; ++i) {
      T acc = B[i + (size_t)j * nr];
      for (int k = j + 1; k < i; ++k) acc += B[i + (size_t)k * nr] * X[k + j * w];
      X[i + j * w] = -acc;
    }
  }
  __syncthreads();
  for (int e = tid; e < w * w; e += nt) {
    const int i = e % w, j = e / w;
    if (i > j) B[i + (size_t)j * nr] = c.Binv[i + j * w];
  }
  __syncthreads();
  lap(PH_SN_INVERSE);
  T *Ls = c.L + r0.w;
  for (int e = tid; e < nr * w; e += nt) {
    T v = B[e];
    if (!(v == v) || isinf((double)v)) atomicOr(c.status, ST_NONFINITE);
    Ls[e] = v;
  }
  for (int m = tid; m < w; m += nt) {
    c.D[c0 + m] = c.Dsm[m];
    c.D[c.N + c0 + m] = c.Esm[m];
    c.lperm[c0 + m] = c.lp[m];
  }
  if (tid == 0) c.piv[s] = pivoted ? 1 : 0;
  __syncthreads();
  lap(PH_SN_STORE);
}

// ---- factorization of one supernode (warp scope) -----------------------------
// The steps and the per-entry arithmetic of factor_sn for a supernode of at
// most wcap columns and rcap rows (both <= 32), by warp wi in its own
// scratch: target rows found by a search of the row list held one per lane,
// descendant updates applied in list order (no atomics), the rows below
// permuted in place along the cycles of the pivot order, and the inverse of
// the unit L11 formed in the block's upper triangle (zero otherwise) before
// it replaces L11.
template <class T> __device__ void factor_sn_warp(Ctx<T> &c, int s, int wi) {
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  if (c.cyc && lane == 0) atomicAdd(&c.cyc[PH_SN], 1ull);
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const int *rows = c.ls + r1.x;
  T *B = c.wB + (size_t)wi * c.wcap * c.rcap;
  T *Dw = c.wD + wi * c.wcap, *Ew = c.wE + wi * c.wcap, *wk = c.wwk + wi * 64;
  int *lpw = c.wlp + wi * c.wcap;
  const int myrow = lane < nr ? rows[lane] : -1;
  // position of row r in the row list, -1 when absent (every lane calls)
  auto find = [&](int r) {
    int pos = -1;
    for (int k = 0; k < nr; ++k)
      if (__shfl_sync(FULL, myrow, k) == r) pos = k;
    return pos;
  };
  for (int e = lane; e < nr * w; e += 32) B[e] = T(0);
  __syncwarp();
  // matrix columns (entries of rows >= the column)
  for (int m = 0; m < w; ++m) {
    const int col = c0 + m, j = c.perm[col];
    const int qb = c.Rp[j], qe = c.Rp[j + 1];
    for (int q0 = qb; q0 < qe; q0 += 32) {
      const int qq = q0 + lane;
      const int oi = qq < qe ? c.iperm[c.Rj[qq]] : -1;
      const int pos = find(oi);
      if (qq < qe && oi >= col) {
        if (pos < 0) atomicOr(c.status, ST_BOUNDS);  // not in the row list: corrupted structure
        else B[pos + m * nr] = T(c.Fv[qq]);
      }
    }
  }
  __syncwarp();
  // descendant updates (sub_update_warp's arithmetic, one pair after another)
  for_visible_pairs(c, s, r1.y, r1.z, r1.w, [&](int pq) {
    const int4 pr = c.prec[pq], d0 = c.snrec[2 * pr.x];
    const int lb = pr.y, ub = pr.z;
    const int cd = d0.x, wd = d0.y, nrd = d0.z;
    const int *rd = c.ls + pr.w;
    const T *Ld = c.L + d0.w;
    const T *Dd = c.D + cd, *Ed = c.D + c.N + cd;
    const int md = nrd - lb, nc = ub - lb + 1;
    for (int i0 = 0; i0 < md; i0 += 32) {
      const int i = i0 + lane;
      const int ri = i < md ? rd[lb + i] : -1;
      int ti = find(ri);
      if (i < md && ti < 0) atomicOr(c.status, ST_BOUNDS);
      for (int jj = 0; jj < nc; ++jj) {
        const int tj = rd[lb + jj] - c0;
        if (tj < 0 || tj >= w) {
          if (lane == 0) atomicOr(c.status, ST_BOUNDS);
          continue;
        }
        if (ti < tj) continue;  // lower triangle of the target only (and absent rows)
        T acc = T(0);
        for (int k = 0; k < wd; ++k) {
          const T lik = Ld[lb + i + (size_t)k * nrd];
          const T ek = Ed[k];
          if (ek == T(0) || k + 1 >= wd) {
            acc += lik * Dd[k] * Ld[lb + jj + (size_t)k * nrd];
          } else {
            const T ljk = Ld[lb + jj + (size_t)k * nrd], ljk1 = Ld[lb + jj + (size_t)(k + 1) * nrd];
            const T lik1 = Ld[lb + i + (size_t)(k + 1) * nrd];
            acc += lik * (Dd[k] * ljk + ek * ljk1) + lik1 * (ek * ljk + Dd[k + 1] * ljk1);
            ++k;
          }
        }
        B[ti + tj * nr] -= acc;
      }
    }
    __syncwarp();
  });
  const bool pivoted = bk_factor_warp<T>(B, nr, w, Dw, Ew, lpw, c.status, wk);
  // rows below: lane owns row r; new column j takes old column lpw[j]
  // (cycles of the pivot order, in place), solve with the unit L11^T, scale
  // by D^-1 (panel_rows_warp0's arithmetic)
  for (int rb0 = w; rb0 < nr; rb0 += 32) {
    const int r = rb0 + lane;
    if (r < nr) {
      T *br = B + r;
      if (pivoted) {
        unsigned done = 0u;
        for (int j0 = 0; j0 < w; ++j0) {
          if ((done >> j0) & 1u) continue;
          const T first = br[(size_t)j0 * nr];
          int j = j0;
          for (int guard = 0; guard < w; ++guard) {
            done |= 1u << j;
            const int src = lpw[j];
            if (src == j0 || src < 0 || src >= w) {
              br[(size_t)j * nr] = first;
              break;
            }
            br[(size_t)j * nr] = br[(size_t)src * nr];
            j = src;
          }
        }
      }
      for (int j = 0; j < w; ++j) {
        T x = br[(size_t)j * nr];
        for (int t = 0; t < j; ++t) x -= br[(size_t)t * nr] * B[j + (size_t)t * nr];
        br[(size_t)j * nr] = x;
      }
      for (int j = 0; j < w; ++j) {
        if (Ew[j] == T(0) || j + 1 >= w) {
          br[(size_t)j * nr] = br[(size_t)j * nr] * (T(1) / Dw[j]);
        } else {
          const T e = Ew[j];
          const T inv = T(1) / (Dw[j] * Dw[j + 1] - e * e);
          const T x1 = br[(size_t)j * nr], x2 = br[(size_t)(j + 1) * nr];
          br[(size_t)j * nr] = (x1 * Dw[j + 1] - x2 * e) * inv;
          br[(size_t)(j + 1) * nr] = (x2 * Dw[j] - x1 * e) * inv;
          ++j;
        }
      }
    }
  }
  __syncwarp();
  // inverse of the unit L11: X(i, j), i > j, at B[j + i nr] (lane j owns row j
  // of the upper triangle), then moved below the diagonal
  if (lane < w) {
    const int j = lane;
    for (int i = j + 1; i < w; ++i) {
      T acc = B[i + (size_t)j * nr];
      for (int k = j + 1; k < i; ++k) acc += B[i + (size_t)k * nr] * B[j + (size_t)k * nr];
      B[j + (size_t)i * nr] = -acc;
    }
  }
  __syncwarp();
  for (int e = lane; e < w * w; e += 32) {
    const int i = e % w, j = e / w;
    if (i > j) B[i + (size_t)j * nr] = B[j + (size_t)i * nr];
  }
  __syncwarp();
  for (int e = lane; e < w * w; e += 32) {
    const int i = e % w, j = e / w;
    if (i > j) B[j + (size_t)i * nr] = T(0);
  }
  __syncwarp();
  T *Ls = c.L + r0.w;
  for (int e = lane; e < nr * w; e += 32) {
    const T v = B[e];
    if (!(v == v) || isinf((double)v)) atomicOr(c.status, ST_NONFINITE);
    Ls[e] = v;
  }
  for (int m = lane; m < w; m += 32) {
    c.D[c0 + m] = Dw[m];
    c.D[c.N + c0 + m] = Ew[m];
    c.lperm[c0 + m] = lpw[m];
  }
  if (lane == 0) c.piv[s] = pivoted ? 1 : 0;
  __syncwarp();
}

// Factor the supernodes of mlist (ascending ids: children before parents,
// the reference's order of mod_indices), then fold the pivots into the row
// lists of the descendants (row_reordering, Sym_BLAS.cpp:327-490) and into
// the ordering (reorder_matrix, linear_solver_wrapper.cpp:1432-1460).
// Level-parallel form: supernodes of one level of the tree are independent
// (each reads only descendants on lower levels and writes only itself), so
// per level the first WF_WARPS warps take the marked supernodes that fit a
// warp, in turn by their rank among the level's marked supernodes, and the
// CTA factors the rest one at a time.  A refactorization of one or two paths
// to the root (at most 2 nlev supernodes, the active-set iterations) keeps
// the CTA path throughout: its supernodes are the widest, with the most
// descendant updates, which the CTA path spreads over every warp.
template <class T> __device__ void factor_marked(Ctx<T> &c) {
  const int m = *c.nmark;
  if (c.wf && m > 2 * c.nlev) {
    const unsigned FULL = 0xffffffffu;
    const int wi = warp_id(), lane = lane_id(), nwf = min(num_warps(), WF_WARPS);
    auto fits = [&](int s) { return c.snrec[2 * s].y <= c.wcap && c.snrec[2 * s].z <= c.rcap; };
    for (int l = 0; l < c.nlev; ++l) {
      // every warp counts the level's supernodes the same way (uniform over the CTA)
      int nfit = 0;
      bool big = false;
      for (int t0 = 0; t0 < m; t0 += 32) {
        const int t = t0 + lane;
        const int s = t < m ? c.mlist[t] : -1;
        const bool at = s >= 0 && c.lev[s] == l;
        nfit += __popc(__ballot_sync(FULL, at && fits(s)));
        big = big || __any_sync(FULL, at && !fits(s));
      }
      if (nfit > 0 && wi < nwf) {
        int seen = 0;
        for (int t0 = 0; t0 < m; t0 += 32) {
          const int t = t0 + lane;
          const int s = t < m ? c.mlist[t] : -1;
          unsigned bal = __ballot_sync(FULL, s >= 0 && c.lev[s] == l && fits(s));
          while (bal) {
            const int b = __ffs(bal) - 1;
            bal &= bal - 1u;
            const int sb = __shfl_sync(FULL, s, b);
            if (seen++ % nwf == wi) factor_sn_warp(c, sb, wi);
          }
        }
      }
      if (nfit > 0) __syncthreads();
      if (big)
        for (int t = 0; t < m; ++t) {
          const int s = c.mlist[t];
          if (c.lev[s] == l && !fits(s)) factor_sn(c, s);
        }
    }
  } else {
    for (int t = 0; t < m; ++t) factor_sn(c, c.mlist[t]);
  }
  BQ_T0(c);
  // renaming: rows of descendants that fall into a pivoted supernode
  for (int t = 0; t < m; ++t) {
    const int s = c.mlist[t];
    if (!c.piv[s]) continue;
    const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
    const int c0 = r0.x, w = r0.y;
    // inverse of the local pivot order: old local position -> new position
    for (int q = threadIdx.x; q < w; q += blockDim.x) c.lp[c.lperm[c0 + q]] = q;
    __syncthreads();
    for (int pq = r1.y; pq < r1.w; ++pq) {
      const int4 pr = c.prec[pq];
      int *rd = c.ls + pr.w;
      for (int i = pr.y + threadIdx.x; i <= pr.z; i += blockDim.x) {
        const int o = rd[i] - c0;
        if (o >= 0 && o < w) rd[i] = c0 + c.lp[o];
        else atomicOr(c.status, ST_BOUNDS);
      }
    }
    // composed ordering: new position q holds the column that was at lperm[q]
    // (old values staged in the free row map)
    for (int q = threadIdx.x; q < w; q += blockDim.x) c.map[q] = c.perm[c0 + c.lperm[c0 + q]];
    __syncthreads();
    for (int q = threadIdx.x; q < w; q += blockDim.x) c.perm[c0 + q] = c.map[q];
    __syncthreads();
    for (int q = threadIdx.x; q < w; q += blockDim.x) c.iperm[c.perm[c0 + q]] = c0 + q;
    __syncthreads();
  }
  for (int t = threadIdx.x; t < m; t += blockDim.x) c.mark[c.mlist[t]] = 0;
  __syncthreads();
  if (threadIdx.x == 0) *c.nmark = 0;
  __syncthreads();
  BQ_T1(c, PH_RENAME);
}

// ---- triangular solves (factor order, vector in shared memory) ---------------
// Forward step of one supernode (reference H2LeveledBlockedLsolve,
// Triangular_BCSC.cpp:378-446): x_s <- L11^-1 x_s through the stored inverse,
// then the rows below push -L21 x_s into their (ancestor) entries; pushes of
// supernodes of the same level may meet, so they are atomic, as in the
// reference's threaded solve (:435).  Wide levels: a thread per supernode,
// narrow levels: a warp per supernode.
template <class T> __device__ void fwd_thread(Ctx<T> &c, int s) {
  T *x = c.xs;
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const T *Ls = c.L + r0.w;
  const int *rows = c.ls + r1.x;
  for (int i = w - 1; i > 0; --i) {  // bottom-up: row i reads x_j, j < i, not yet replaced
    T acc = x[c0 + i];
    for (int j = 0; j < i; ++j) acc += Ls[i + (size_t)j * nr] * x[c0 + j];
    x[c0 + i] = acc;
  }
#pragma unroll 4
  for (int r = w; r < nr; ++r) {
    T y = T(0);
    for (int k = 0; k < w; ++k) y += Ls[r + (size_t)k * nr] * x[c0 + k];
    const int rr = rows[r];
    if ((unsigned)rr < (unsigned)c.N) atomicAdd(&x[rr], -y);
  }
}

template <class T> __device__ void fwd_warp(Ctx<T> &c, int s) {
  T *x = c.xs;
  const int lane = lane_id();
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const T *Ls = c.L + r0.w;
  const int *rows = c.ls + r1.x;
  // x_s <- L11^-1 x_s: lanes form rows of the product, then write; chunks
  // of 32 rows from the bottom (a chunk reads only rows above it)
  for (int i0 = ((w - 1) / 32) * 32; i0 >= 0; i0 -= 32) {
    const int i = i0 + lane;
    T acc = T(0);
    if (i < w) {
      acc = x[c0 + i];
      for (int j = 0; j < i; ++j) acc += Ls[i + (size_t)j * nr] * x[c0 + j];
    }
    __syncwarp();
    if (i < w) x[c0 + i] = acc;
    __syncwarp();
  }
  for (int r = w + lane; r < nr; r += 32) {
    T y = T(0);
    for (int k = 0; k < w; ++k) y += Ls[r + (size_t)k * nr] * x[c0 + k];
    const int rr = rows[r];
    if ((unsigned)rr < (unsigned)c.N) atomicAdd(&x[rr], -y);
  }
  __syncwarp();
}

// Backward (Triangular_BCSC.cpp:534-600): x1 -= L21^T x(rows below), then
// x1 <- L11^-T x1 through the stored inverse.
template <class T> __device__ void bwd_thread(Ctx<T> &c, int s) {
  T *x = c.xs;
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const int *rows = c.ls + r1.x;
  const T *Ls = c.L + r0.w;
  for (int j = 0; j < w; ++j) {
    T acc = T(0);
#pragma unroll 4
    for (int r = w; r < nr; ++r) {
      const int rr = rows[r];
      if ((unsigned)rr < (unsigned)c.N) acc += Ls[r + (size_t)j * nr] * x[rr];
    }
    x[c0 + j] -= acc;
  }
  // top-down: entry j reads x_i, i > j, not yet replaced
  for (int j = 0; j + 1 < w; ++j) {
    T acc = x[c0 + j];
    for (int i = j + 1; i < w; ++i) acc += Ls[i + (size_t)j * nr] * x[c0 + i];
    x[c0 + j] = acc;
  }
}

template <class T> __device__ void bwd_warp(Ctx<T> &c, int s) {
  T *x = c.xs;
  const int lane = lane_id();
  const int4 r0 = c.snrec[2 * s], r1 = c.snrec[2 * s + 1];
  const int c0 = r0.x, w = r0.y, nr = r0.z;
  const int *rows = c.ls + r1.x;
  const T *Ls = c.L + r0.w;
  for (int j = 0; j < w; ++j) {
    T acc = T(0);
    for (int r = w + lane; r < nr; r += 32) {
      const int rr = rows[r];
      if ((unsigned)rr < (unsigned)c.N) acc += Ls[r + (size_t)j * nr] * x[rr];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) x[c0 + j] -= acc;
  }
  __syncwarp();
  // x_s <- L11^-T x_s: lanes form entries of the product, chunks of 32 from the top
  for (int j0 = 0; j0 < w; j0 += 32) {
    const int j = j0 + lane;
    T acc = T(0);
    if (j < w) {
      acc = x[c0 + j];
      for (int i = j + 1; i < w; ++i) acc += Ls[i + (size_t)j * nr] * x[c0 + i];
    }
    __syncwarp();
    if (j < w) x[c0 + j] = acc;
    __syncwarp();
  }
}

// x <- (L D L^T)^-1 x on the visible part, in the factor's order.  Per
// level, small supernodes take a thread each and big ones a warp each, in
// the same pass (supernodes of one level are independent).
template <class T> __device__ void ldlt_solve_smem(Ctx<T> &c) {
  const int nw = num_warps();
  {
    BQ_T0(c);
    for (int l = 0; l < c.nlev; ++l) {
      const int a = c.vlvl[l], m = c.vmid[l], b = c.vlvl[l + 1];
      for (int q = a + threadIdx.x; q < m; q += blockDim.x) fwd_thread(c, c.vlist[q]);
      for (int q = m + warp_id(); q < b; q += nw) fwd_warp(c, c.vlist[q]);
      __syncthreads();
    }
    BQ_T1(c, PH_FWD_WIDE);
  }
  {
    BQ_T0(c);
    // D solve: 1x1 by division, 2x2 by Cramer's rule (blocked_2by2_solver, Sym_BLAS.cpp:492-529)
    for (int i = threadIdx.x; i < c.N; i += blockDim.x) {
      if (!visible(c, c.col2sup[i])) continue;
      if (i > 0 && c.D[c.N + i - 1] != T(0)) continue;  // second column of a 2x2 block
      const T e = i + 1 < c.N ? c.D[c.N + i] : T(0);
      if (e == T(0)) {
        c.xs[i] = c.xs[i] / c.D[i];
      } else {
        const T d1 = c.D[i], d2 = c.D[i + 1];
        const T inv = T(1) / (d1 * d2 - e * e);
        const T x1 = c.xs[i], x2 = c.xs[i + 1];
        c.xs[i] = (x1 * d2 - x2 * e) * inv;
        c.xs[i + 1] = (x2 * d1 - x1 * e) * inv;
      }
    }
    __syncthreads();
    BQ_T1(c, PH_DIAG);
  }
  BQ_T0(c);
  for (int l = c.nlev - 1; l >= 0; --l) {
    const int a = c.vlvl[l], m = c.vmid[l], b = c.vlvl[l + 1];
    for (int q = a + threadIdx.x; q < m; q += blockDim.x) bwd_thread(c, c.vlist[q]);
    for (int q = m + warp_id(); q < b; q += nw) bwd_warp(c, c.vlist[q]);
    __syncthreads();
  }
  BQ_T1(c, PH_BWD);
}

// Visible supernodes grouped by level (after every change of the active set):
// per level the small ones, then the big ones.
template <class T> __device__ void build_vlist(Ctx<T> &c) {
  const int L1 = c.nlev + 1;
  for (int l = threadIdx.x; l < 2 * L1; l += blockDim.x) c.vfill[l] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < c.ns; s += blockDim.x)
    if (c.vis[s]) atomicAdd(&c.vfill[c.lev[s] + (c.sn_big[s] ? L1 : 0)], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int l = 0; l < c.nlev; ++l) {
      c.vlvl[l] = acc;
      acc += c.vfill[l];
      c.vmid[l] = acc;
      acc += c.vfill[L1 + l];
      c.vfill[l] = c.vlvl[l];     // next free position of the small ones
      c.vfill[L1 + l] = c.vmid[l];  // and of the big ones
    }
    c.vlvl[c.nlev] = acc;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < c.ns; s += blockDim.x)
    if (c.vis[s]) c.vlist[atomicAdd(&c.vfill[c.lev[s] + (c.sn_big[s] ? L1 : 0)], 1)] = s;
  __syncthreads();
}

// out = M^-1 v (original numbering; hidden rows give zero).  Vectors in
// global memory, the solve in shared memory.
template <class T, class VI, class VO> __device__ void precond(Ctx<T> &c, const VI *v, VO *out) {
  BQ_T0(c);
  const long long tg0 = c.cyc ? clock64() : 0;
  for (int i = threadIdx.x; i < c.N; i += blockDim.x) c.xs[i] = visible(c, c.col2sup[i]) ? T(v[c.perm[i]]) : T(0);
  __syncthreads();
  if (c.cyc && threadIdx.x == 0) c.cyc[PH_GATHER] += (unsigned long long)(clock64() - tg0);
  ldlt_solve_smem(c);
  const long long tg1 = c.cyc ? clock64() : 0;
  for (int i = threadIdx.x; i < c.N; i += blockDim.x) out[c.perm[i]] = VO(c.xs[i]);
  __syncthreads();
  if (c.cyc && threadIdx.x == 0) c.cyc[PH_GATHER] += (unsigned long long)(clock64() - tg1);
  BQ_T1(c, PH_PRECOND);
}

// y = K x with the refinement values (original numbering).
template <class T> __device__ void spmv_ref(const Ctx<T> &c, const double *x, double *y) {
  BQ_T0(c);
  for (int i = threadIdx.x; i < c.N; i += blockDim.x) {
    double acc = 0.0;
    for (int qq = c.Rp[i]; qq < c.Rp[i + 1]; ++qq) acc += c.Rv[qq] * x[c.Rj[qq]];
    y[i] = acc;
  }
  __syncthreads();
  BQ_T1(c, PH_SPMV);
}

template <class T> __device__ double dot(const Ctx<T> &c, const double *a, const double *b) {
  double s = 0.0;
  for (int i = threadIdx.x; i < c.N; i += blockDim.x) s += a[i] * b[i];
  return block_sum(s, c.red);
}

// ---- refinement (reference pmgmres_ldlt_auto, src/gmres/mgmres.cpp:1015-1211)
struct GmresSmall {
  double h[MR_CAP + 1][MR_CAP], cs[MR_CAP + 1], sn[MR_CAP + 1], g[MR_CAP + 1], y[MR_CAP + 1];
  double scal[4];
};

// Solves K x = b (x holds the preconditioned solution on entry).  flexible:
// right-preconditioned FGMRES with stored directions Z (Saad 1993) -- the
// residual it minimises is the FP64 b - Kx itself; else the reference's
// left-preconditioned GMRES.  adaptive: stop once the residual estimate is
// below rtol * ||b||; else the reference's rule (rho <= tol_rel * rho0 and
// rho <= tol_abs).  Returns the Krylov steps taken.
template <class T>
__device__ int refine(Ctx<T> &c, const double *b, double *x, int itr_max, int mr, bool flexible, bool adaptive,
                      double rtol, double tol_abs, double tol_rel, GmresSmall &gs) {
  if (itr_max <= 0 || mr <= 0) return 0;
  mr = min(mr, MR_CAP);
  const int N = c.N;
  const double delta = 1.0e-03;
  double *r = c.r, *V = c.V;
  double rho = 0.0, rho_tol = 0.0, stop_abs = tol_abs;
  int used = 0;
  if (adaptive) {
    const double nb = sqrt(dot(c, b, b));
    stop_abs = rtol * nb;
  }
  for (int itr = 0; itr < itr_max; ++itr) {
    spmv_ref(c, x, r);
    for (int i = threadIdx.x; i < N; i += blockDim.x) r[i] = b[i] - r[i];
    __syncthreads();
    if (!flexible) precond(c, r, r);
    rho = sqrt(dot(c, r, r));
    if (adaptive ? rho <= stop_abs : rho < tol_abs) return used;
    if (itr == 0) rho_tol = rho * tol_rel;
    for (int i = threadIdx.x; i < N; i += blockDim.x) V[i] = r[i] / rho;
    if (threadIdx.x == 0) {
      gs.g[0] = rho;
      for (int i = 1; i <= mr; ++i) gs.g[i] = 0.0;
      for (int i = 0; i <= mr; ++i)
        for (int j = 0; j < mr; ++j) gs.h[i][j] = 0.0;
    }
    __syncthreads();
    int k_copy = 0;
    bool stop = false;
    for (int k = 0; k < mr; ++k) {
      k_copy = k;
      double *vk = V + (size_t)k * N, *vk1 = V + (size_t)(k + 1) * N;
      if (flexible) {
        T *zk = c.Z + (size_t)k * N;
        precond(c, vk, zk);
        // A z_k in FP64 (z widened)
        for (int i = threadIdx.x; i < N; i += blockDim.x) c.w[i] = (double)zk[i];
        __syncthreads();
        spmv_ref(c, c.w, vk1);
      } else {
        spmv_ref(c, vk, vk1);
        precond(c, vk1, vk1);
      }
      const double av = sqrt(dot(c, vk1, vk1));
      for (int j = 0; j <= k; ++j) {
        const double hj = dot(c, vk1, V + (size_t)j * N);
        for (int i = threadIdx.x; i < N; i += blockDim.x) vk1[i] -= hj * V[(size_t)j * N + i];
        if (threadIdx.x == 0) gs.h[j][k] = hj;
        __syncthreads();
      }
      double hk1 = sqrt(dot(c, vk1, vk1));
      if ((av + delta * hk1) == av) {
        for (int j = 0; j <= k; ++j) {
          const double ht = dot(c, vk1, V + (size_t)j * N);
          for (int i = threadIdx.x; i < N; i += blockDim.x) vk1[i] -= ht * V[(size_t)j * N + i];
          if (threadIdx.x == 0) gs.h[j][k] += ht;
          __syncthreads();
        }
        hk1 = sqrt(dot(c, vk1, vk1));
      }
      if (hk1 != 0.0)
        for (int i = threadIdx.x; i < N; i += blockDim.x) vk1[i] = vk1[i] / hk1;
      if (threadIdx.x == 0) {
        gs.h[k + 1][k] = hk1;
        if (0 < k) {
          for (int j = 0; j < k; ++j) {  // previous Givens rotations
            const double g1 = gs.cs[j] * gs.h[j][k] - gs.sn[j] * gs.h[j + 1][k];
            const double g2 = gs.sn[j] * gs.h[j][k] + gs.cs[j] * gs.h[j + 1][k];
            gs.h[j][k] = g1;
            gs.h[j + 1][k] = g2;
          }
        }
        const double mu = sqrt(gs.h[k][k] * gs.h[k][k] + gs.h[k + 1][k] * gs.h[k + 1][k]);
        gs.scal[0] = mu;
        if (mu != 0.0) {
          gs.cs[k] = gs.h[k][k] / mu;
          gs.sn[k] = -gs.h[k + 1][k] / mu;
          gs.h[k][k] = gs.cs[k] * gs.h[k][k] - gs.sn[k] * gs.h[k + 1][k];
          gs.h[k + 1][k] = 0.0;
          const double g1 = gs.cs[k] * gs.g[k] - gs.sn[k] * gs.g[k + 1];
          const double g2 = gs.sn[k] * gs.g[k] + gs.cs[k] * gs.g[k + 1];
          gs.g[k] = g1;
          gs.g[k + 1] = g2;
        }
      }
      __syncthreads();
      if (gs.scal[0] == 0.0) return used;
      rho = fabs(gs.g[k + 1]);
      used++;
      stop = adaptive ? rho <= stop_abs : (rho <= rho_tol && rho <= tol_abs);
      if (stop) break;
    }
    const int k = k_copy;
    if (gs.h[k][k] == 0.0) return used;
    if (threadIdx.x == 0) {
      gs.y[k] = gs.g[k] / gs.h[k][k];
      for (int i = k - 1; 0 <= i; i--) {
        double yi = gs.g[i];
        for (int j = i + 1; j < k + 1; j++) yi = yi - gs.h[i][j] * gs.y[j];
        gs.y[i] = yi / gs.h[i][i];
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      double acc = 0.0;
      if (flexible)
        for (int j = 0; j <= k; ++j) acc += (double)c.Z[(size_t)j * N + i] * gs.y[j];
      else
        for (int j = 0; j <= k; ++j) acc += V[(size_t)j * N + i] * gs.y[j];
      x[i] += acc;
    }
    __syncthreads();
    if (stop) break;
  }
  return used;
}

// ---- NASOQ on one problem ------------------------------------------------------
// Marks the supernodes on the elimination-tree path from supernode s to the
// root and appends them to mlist (the reference marks the visible ones of its
// edited tree, which are a subset; refactoring an unchanged supernode
// reproduces it).  Thread 0 only.
template <class T> __device__ void mark_path(Ctx<T> &c, int s) {
  for (; s >= 0; s = c.sparent[s])
    if (!c.mark[s]) {
      c.mark[s] = 1;
      c.mlist[(*c.nmark)++] = s;
    }
}

// KKT edit of constraint k (reference edit_kkt -> add_del_matrix_qp,
// linear_solver_wrapper.cpp:1020-1137): the constraint's entries become
// visible / hidden in both value copies and in the descendant masks of its
// targets, and the paths of its column and of its variables are marked for
// the next partial refactorization.  Thread 0 only.
template <class T> __device__ void edit_constraint(Ctx<T> &c, int k, bool add) {
  c.act[k] = add ? 1 : 0;
  c.vis[c.con_sn[k]] = add ? 1 : 0;
  for (int e = c.bt_ptr[k]; e < c.bt_ptr[k + 1]; ++e) {
    const int qq = c.bt_rpos[e];
    const double v = add ? c.kv[c.bt_q[e]] : 0.0;
    c.Fv[qq] = v;
    c.Rv[qq] = v;
  }
  const int row = c.base + k;
  for (int qq = c.Rp[row]; qq < c.Rp[row + 1]; ++qq)
    if (c.Rj[qq] != row) {
      const double v = add ? c.kv[c.Rq[qq]] : 0.0;
      c.Fv[qq] = v;
      c.Rv[qq] = v;
    }
  for (int e = c.con_ptr[k]; e < c.con_ptr[k + 1]; ++e) {
    const int tg = c.con_tgt[2 * e], bit = c.con_tgt[2 * e + 1];
    if (bit < 64) {
      if (add) c.cmask[tg] |= 1ull << bit;
      else c.cmask[tg] &= ~(1ull << bit);
    }
  }
  mark_path(c, c.con_sn[k]);
  for (int e = c.bt_ptr[k]; e < c.bt_ptr[k + 1]; ++e) mark_path(c, c.col2sup[c.iperm[c.bt_var[e]]]);
}

// Marks every supernode (visible ones only when `only_visible`), in
// ascending order.
template <class T> __device__ void mark_all(Ctx<T> &c, bool only_visible) {
  int base = 0;
  for (int q0 = 0; q0 < c.ns; q0 += blockDim.x) {
    const int q = q0 + threadIdx.x;
    const int f = (q < c.ns && (!only_visible || c.vis[q])) ? 1 : 0;
    if (q < c.ns) c.mark[q] = (uint8_t)f;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int wpre = __popc(bal & ((1u << lane_id()) - 1u));
    if (lane_id() == 0) c.redi[warp_id()] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int t = 0; t < num_warps(); ++t) {
      if (t < warp_id()) before += c.redi[t];
      total += c.redi[t];
    }
    if (f) c.mlist[base + before + wpre] = q;
    base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *c.nmark = base;
  __syncthreads();
}

// Sorts mlist ascending (children before parents).  Thread 0; the lists of
// partial refactorizations are a few tree paths long.
template <class T> __device__ void sort_mlist(Ctx<T> &c) {
  if (threadIdx.x == 0) {
    const int m = *c.nmark;
    for (int i = 1; i < m; ++i) {
      const int v = c.mlist[i];
      int j = i - 1;
      while (j >= 0 && c.mlist[j] > v) {
        c.mlist[j + 1] = c.mlist[j];
        --j;
      }
      c.mlist[j + 1] = v;
    }
  }
  __syncthreads();
}

// Slot state of a problem whose group shares one factorization: the factor,
// its pivoting state and both value copies of K with every inequality
// hidden, copied from the group's base slot; visibility likewise.
template <class T> __device__ void copy_base(Ctx<T> &c, const unsigned char *bs, const BSlot &L, const BPat &pt) {
  const int tid = threadIdx.x, nt = blockDim.x, N = c.N;
  const T *bL = reinterpret_cast<const T *>(bs + L.o_L);
  const T *bD = reinterpret_cast<const T *>(bs + L.o_D);
  const int *bls = reinterpret_cast<const int *>(bs + L.o_ls);
  const int *bperm = reinterpret_cast<const int *>(bs + L.o_perm);
  const int *biperm = reinterpret_cast<const int *>(bs + L.o_iperm);
  const int *blperm = reinterpret_cast<const int *>(bs + L.o_lperm);
  const double *bF = reinterpret_cast<const double *>(bs + L.o_Fv);
  const double *bR = reinterpret_cast<const double *>(bs + L.o_Rv);
  const unsigned long long *bmask = reinterpret_cast<const unsigned long long *>(bs + L.o_cmask);
  for (int i = tid; i < pt.xsize; i += nt) c.L[i] = bL[i];
  for (int i = tid; i < 2 * N; i += nt) c.D[i] = bD[i];
  for (int i = tid; i < pt.ssize; i += nt) c.ls[i] = bls[i];
  for (int i = tid; i < N; i += nt) {
    c.perm[i] = bperm[i];
    c.iperm[i] = biperm[i];
    c.lperm[i] = blperm[i];
  }
  for (int i = tid; i < c.nnzR; i += nt) {
    c.Fv[i] = bF[i];
    c.Rv[i] = bR[i];
  }
  for (int s = tid; s < c.ns; s += nt) {
    c.piv[s] = bs[L.o_piv + s];
    c.cmask[s] = bmask[s];
    c.mark[s] = 0;
    c.vis[s] = c.sn_con[s] < 0 ? 1 : 0;
  }
  if (tid == 0) *c.nmark = 0;
  __syncthreads();
}

// Visibility, descendant masks and both value copies of K from the active set.
template <class T> __device__ void load_state(Ctx<T> &c) {
  for (int s = threadIdx.x; s < c.ns; s += blockDim.x) {
    const int k = c.sn_con[s];
    c.vis[s] = (k < 0 || c.act[k]) ? 1 : 0;
    c.cmask[s] = 0ull;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < c.mineq; k += blockDim.x)
    if (c.act[k])
      for (int e = c.con_ptr[k]; e < c.con_ptr[k + 1]; ++e) {
        const int bit = c.con_tgt[2 * e + 1];
        if (bit < 64) atomicOr(c.cmask + c.con_tgt[2 * e], 1ull << bit);
      }
  for (int qq = threadIdx.x; qq < c.nnzR; qq += blockDim.x) {
    const int vq = c.Rq[qq];
    c.Fv[qq] = fact_val(c, vq);
    c.Rv[qq] = ref_val(c, vq);
  }
  __syncthreads();
}

}  // namespace

template <class T>
__global__ void __launch_bounds__(BT_MAX_THREADS) k_nasoq_batch(BArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ int s_status, s_prob;
  __shared__ GmresSmall gs;
  __shared__ int s_int[8];
  __shared__ double s_dbl[8];
  __shared__ int s_nmark;
  __shared__ Ctx<T> sc;  // the problem's context, read by every thread
  __shared__ unsigned long long s_cyc[PH_N];
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid < PH_N) s_cyc[tid] = 0;
  // shared-memory carve-up (sizes from the largest pattern of the batch)
  auto up16 = [](size_t v) { return (v + 15) / 16 * 16; };
  unsigned char *sp = smem;
  int *map = reinterpret_cast<int *>(sp);
  sp += up16((size_t)a.N_max * sizeof(int));
  T *xs = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.N_max * sizeof(T));
  T *Bm = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.nr_max * a.w_max * sizeof(T));
  T *rowbuf = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.w_max * 32 * sizeof(T));
  T *Dsm = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.w_max * sizeof(T));
  T *Esm = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.w_max * sizeof(T));
  int *lp = reinterpret_cast<int *>(sp);
  sp += up16((size_t)a.w_max * sizeof(int));
  T *Binv = reinterpret_cast<T *>(sp);
  sp += up16((size_t)a.w_max * a.w_max * sizeof(T));
  int *vlvl = reinterpret_cast<int *>(sp);
  sp += up16((size_t)(a.nlev_max + 1) * sizeof(int));
  int *vmid = reinterpret_cast<int *>(sp);
  sp += up16((size_t)(a.nlev_max + 1) * sizeof(int));
  int *vfill = reinterpret_cast<int *>(sp);
  sp += up16((size_t)2 * (a.nlev_max + 1) * sizeof(int));
  uint8_t *vis = sp;
  sp += up16((size_t)a.ns_max);
  uint8_t *act = sp;
  sp += up16((size_t)a.mi_max);
  const int wcap = min(a.w_max, 32), rcap = min(a.nr_max, 32);
  T *wB = nullptr, *wD = nullptr, *wE = nullptr, *wwk = nullptr;
  int *wlp = nullptr;
  if (a.warp_factor) {
    wB = reinterpret_cast<T *>(sp);
    sp += up16((size_t)WF_WARPS * wcap * rcap * sizeof(T));
    wD = reinterpret_cast<T *>(sp);
    sp += up16((size_t)WF_WARPS * wcap * sizeof(T));
    wE = reinterpret_cast<T *>(sp);
    sp += up16((size_t)WF_WARPS * wcap * sizeof(T));
    wlp = reinterpret_cast<int *>(sp);
    sp += up16((size_t)WF_WARPS * wcap * sizeof(int));
    wwk = reinterpret_cast<T *>(sp);
    sp += up16((size_t)WF_WARPS * 64 * sizeof(T));
  }
  unsigned char *stage = sp;  // the factor and row lists of a problem that fits

  unsigned char *const own_slot = a.slots + (size_t)blockIdx.x * a.slot.bytes;
  const bool build_bases = a.mode == 1;
  for (;;) {
    if (tid == 0) {
      const int qi = atomicAdd(a.head, 1);
      if (build_bases) s_prob = qi < a.nbase ? qi : -1;  // a group
      else s_prob = qi < a.nprob ? a.order[qi] : -1;
      s_status = 0;
      s_nmark = 0;
    }
    __syncthreads();
    if (s_prob < 0) break;
    // mode 1: the group's shared factorization is built in its base slot,
    // for the group's representative problem
    const int grp = build_bases ? s_prob : -1;
    const int pi = build_bases ? a.base_rep[grp] : s_prob;
    unsigned char *const slot = build_bases ? a.bases + (size_t)grp * a.slot.bytes : own_slot;
    const BProb &P = a.probs[pi];
    const BPat &pt = a.pats[P.pat];
    Ctx<T> &c = sc;
    if (tid == 0) {
      const int *ip = a.ipool;
      c.n = pt.n;
      c.meq = pt.meq;
      c.mineq = pt.mineq;
      c.N = pt.N;
      c.base = pt.base;
      c.ns = pt.ns;
      c.nlev = pt.nlev;
      c.nnzR = pt.nnzR;
      c.cmask_ok = pt.cmask_ok;
      c.super = ip + pt.o_super;
      c.sparent = ip + pt.o_sparent;
      c.col2sup = ip + pt.o_col2sup;
      c.lpi = ip + pt.o_lpi;
      c.lpx = ip + pt.o_lpx;
      c.lvl_ptr = ip + pt.o_lvl_ptr;
      c.lvl_sn = ip + pt.o_lvl_sn;
      c.lev = ip + pt.o_lev;
      c.Rp = ip + pt.o_Rp;
      c.Rj = ip + pt.o_Rj;
      c.Rq = ip + pt.o_Rq;
      c.ent = ip + pt.o_ent;
      c.bt_ptr = ip + pt.o_bt_ptr;
      c.bt_var = ip + pt.o_bt_var;
      c.bt_q = ip + pt.o_bt_q;
      c.bt_rpos = ip + pt.o_bt_rpos;
      c.sn_con = ip + pt.o_sn_con;
      c.con_sn = ip + pt.o_con_sn;
      c.eq_ptr = ip + pt.o_eq_ptr;
      c.eq_var = ip + pt.o_eq_var;
      c.eq_q = ip + pt.o_eq_q;
      c.snrec = reinterpret_cast<const int4 *>(ip + pt.o_snrec);
      c.prec = reinterpret_cast<const int4 *>(ip + pt.o_prec);
      c.con_ptr = ip + pt.o_con_ptr;
      c.con_tgt = ip + pt.o_con_tgt;
      c.sn_big = reinterpret_cast<const uint8_t *>(ip + pt.o_sn_big);
      c.kv = a.dpool + P.o_kv;
      c.q = a.dpool + P.o_q;
      c.bq = a.dpool + P.o_b;
      c.dq = a.dpool + P.o_d;
      c.pert = reinterpret_cast<const uint8_t *>(a.dpool) + P.o_pert;
      c.reg = P.reg;
      c.reg32 = P.reg32;
      // the factor and the row lists live in shared memory when they fit
      const size_t lbytes = ((size_t)pt.xsize * sizeof(T) + 15) / 16 * 16;
      if (!build_bases && lbytes + (size_t)pt.ssize * sizeof(int) <= (size_t)a.stage_bytes) {
        c.L = reinterpret_cast<T *>(stage);
        c.ls = reinterpret_cast<int *>(stage + lbytes);
      } else {
        c.L = reinterpret_cast<T *>(slot + a.slot.o_L);
        c.ls = reinterpret_cast<int *>(slot + a.slot.o_ls);
      }
      c.D = reinterpret_cast<T *>(slot + a.slot.o_D);
      c.perm = reinterpret_cast<int *>(slot + a.slot.o_perm);
      c.iperm = reinterpret_cast<int *>(slot + a.slot.o_iperm);
      c.lperm = reinterpret_cast<int *>(slot + a.slot.o_lperm);
      c.mark = slot + a.slot.o_mark;
      c.piv = slot + a.slot.o_piv;
      c.alist = reinterpret_cast<int *>(slot + a.slot.o_alist);
      c.vlist = reinterpret_cast<int *>(slot + a.slot.o_vlist);
      c.mlist = reinterpret_cast<int *>(slot + a.slot.o_mlist);
      c.Fv = reinterpret_cast<double *>(slot + a.slot.o_Fv);
      c.Rv = reinterpret_cast<double *>(slot + a.slot.o_Rv);
      c.cmask = reinterpret_cast<unsigned long long *>(slot + a.slot.o_cmask);
      c.rhs = reinterpret_cast<double *>(slot + a.slot.o_rhs);
      c.sol = reinterpret_cast<double *>(slot + a.slot.o_sol);
      c.r = reinterpret_cast<double *>(slot + a.slot.o_r);
      c.w = reinterpret_cast<double *>(slot + a.slot.o_w);
      c.V = reinterpret_cast<double *>(slot + a.slot.o_V);
      c.Z = reinterpret_cast<T *>(slot + a.slot.o_Z);
      c.tmp = reinterpret_cast<double *>(slot + a.slot.o_tmp);
      c.map = map;
      c.xs = xs;
      c.B = Bm;
      c.rowbuf = rowbuf;
      c.Dsm = Dsm;
      c.Esm = Esm;
      c.Binv = Binv;
      c.lp = lp;
      c.wB = wB;
      c.wD = wD;
      c.wE = wE;
      c.wlp = wlp;
      c.wwk = wwk;
      c.wcap = wcap;
      c.rcap = rcap;
      c.wf = a.warp_factor ? 1 : 0;
      c.vis = vis;
      c.act = act;
      c.vlvl = vlvl;
      c.vmid = vmid;
      c.vfill = vfill;
      c.nmark = &s_nmark;
      c.red = red;
      c.redi = redi;
      c.status = &s_status;
      c.cyc = a.prof ? s_cyc : nullptr;
    }
    __syncthreads();
    const long long tp0 = clock64();
    const int *ip = a.ipool;
    double *xv = a.dout + P.o_x, *yv = a.dout + P.o_y, *zv = a.dout + P.o_z;
    int *as_out = a.iout + P.o_as;
    const int n = c.n, meq = c.meq, mineq = c.mineq, N = c.N;
    const bool flexible = sizeof(T) == 4 || a.refine == 1;
    const bool adaptive = a.refine == 1;
    int steps = 0, solves = 0, warm_dropped = 0;

    // ---- set-up: pattern state into the slot (a problem of a group starts
    // from the group's factorization instead, below)
    if (build_bases || P.base < 0) {
      for (int i = tid; i < N; i += nt) {
        const int p0 = ip[pt.o_perm0 + i];
        c.perm[i] = p0;
        c.iperm[p0] = i;
        c.D[i] = T(0);
        c.D[N + i] = T(0);
      }
      for (int i = tid; i < pt.ssize; i += nt) c.ls[i] = ip[pt.o_ls0 + i];
      for (int i = tid; i < pt.xsize; i += nt) c.L[i] = T(0);
      for (int s = tid; s < c.ns; s += nt) {
        c.mark[s] = 0;
        c.piv[s] = 0;
      }
    }
    for (int k = tid; k < mineq; k += nt) c.act[k] = 0;
    __syncthreads();
    if (build_bases) {  // every inequality hidden: the cold start's factorization
      load_state(c);
      build_vlist(c);
      mark_all(c, true);
      factor_marked(c);
      continue;
    }
    const unsigned char *const bslot = P.base >= 0 ? a.bases + (size_t)P.base * a.slot.bytes : nullptr;
    int nact = 0;
    // warm start: proposed active set (constraints listed in as_out), then
    // the equality-constrained solution on it (below)
    const bool warm = P.ws_n >= 0;
    if (warm) {
      for (int t = tid; t < P.ws_n; t += nt) {
        const int k = as_out[t];
        if (k >= 0 && k < mineq) c.act[k] = 1;
      }
      __syncthreads();
    }
    // ---- initial factorization and solution (reference initialize_x,
    // src/nasoq.cpp:448-476): every visible supernode; rhs [-q; b; d on the
    // active rows]
    // Only visible supernodes are factored: a hidden one contributes zeros
    // and is skipped by the solves.  After the first warm round, dropped
    // constraints are hidden by the partial refactorization of their paths.
    bool cold = !warm, full = true;
    for (int round = 0; round < 5; ++round) {
      const long long tf0 = c.cyc ? clock64() : 0;
      if (full && bslot) {
        // the group's cold factorization, then the active rows made visible
        // by partial refactorization of their paths
        copy_base(c, bslot, a.slot, pt);
        if (tid == 0)
          for (int k = 0; k < mineq; ++k)
            if (c.act[k]) edit_constraint(c, k, true);
        __syncthreads();
        sort_mlist(c);
        factor_marked(c);
        build_vlist(c);
      } else if (full) {
        load_state(c);
        build_vlist(c);
        mark_all(c, true);
        factor_marked(c);
      } else {
        sort_mlist(c);
        factor_marked(c);
        build_vlist(c);
      }
      if (c.cyc && tid == 0) c.cyc[PH_INIT_FACTOR] += (unsigned long long)(clock64() - tf0);
      for (int i = tid; i < N; i += nt) {
        double v = 0.0;
        if (i < n) v = -c.q[i];
        else if (i < c.base) v = c.bq[i - n];
        else if (c.act[i - c.base]) v = c.dq[i - c.base];
        c.rhs[i] = v;
      }
      __syncthreads();
      precond(c, c.rhs, c.sol);
      solves++;
      steps += refine(c, c.rhs, c.sol, P.outer, P.inner, flexible, adaptive, a.refine_tol, P.tol_abs, P.tol_rel, gs);
      if (cold) break;
      // a proposed set that makes the KKT matrix singular (dependent
      // constraints): start cold instead
      int bad = 0;
      for (int i = tid; i < N; i += nt)
        if (!isfinite(c.sol[i])) bad++;
      bad = block_sum_int(bad, redi);
      if (bad > 0 || (s_status & (ST_ZERO_PIVOT | ST_NONFINITE))) {
        for (int k = tid; k < mineq; k += nt) c.act[k] = 0;
        __syncthreads();
        if (tid == 0) s_status = 0;
        cold = true;
        full = true;
        __syncthreads();
        continue;
      }
      // drop proposed constraints with negative multipliers, then solve again
      if (tid == 0) {
        int nd = 0;
        for (int k = 0; k < mineq; ++k)
          if (c.act[k] && c.sol[c.base + k] < 0.0) {
            edit_constraint(c, k, false);
            nd++;
          }
        s_int[2] = nd;
      }
      __syncthreads();
      const int ndrop = s_int[2];
      warm_dropped += ndrop;
      if (ndrop == 0) break;
      full = false;
      if (round >= 2) {  // no consistent set after three rounds: cold start
        for (int k = tid; k < mineq; k += nt) c.act[k] = 0;
        if (tid == 0) {
          for (int t = 0; t < *c.nmark; ++t) c.mark[c.mlist[t]] = 0;
          *c.nmark = 0;
        }
        cold = true;
        full = true;
        __syncthreads();
      }
    }
    for (int i = tid; i < n; i += nt) xv[i] = c.sol[i];
    for (int i = tid; i < meq; i += nt) yv[i] = c.sol[n + i];
    for (int k = tid; k < mineq; k += nt) zv[k] = c.act[k] ? c.sol[c.base + k] : 0.0;
    __syncthreads();
    if (tid == 0) {
      for (int k = 0; k < mineq; ++k)
        if (c.act[k]) c.alist[nact++] = k;
      s_int[0] = nact;
    }
    __syncthreads();
    nact = s_int[0];
    if (c.cyc && tid == 0) c.cyc[PH_INIT] += (unsigned long long)(clock64() - tp0);

    // ---- the dual active-set iteration (reference numeric_QP)
    int num_iter = 0, converged = 0, nxt_active = -1, nxt_drop = -1, to_add = 1;
    int typ = 0;  // 0 solve, 1 update (partial refactorization first)
    const double DMAX = DBL_MAX;
    for (int pol = 0;; ++pol) {
    for (;;) {
      if (num_iter > P.max_iter_nas) {
        converged = 0;
        break;
      }
      if (to_add == 1) {
        BQ_T0(c);
        // primal_feasibility (src/nasoq.cpp:787-840): most violated row beyond eps_abs
        int viol = 0;
        double best = P.eps_abs;
        int bi = -1;
        for (int k = tid; k < mineq; k += nt) {
          double t = 0.0;
          for (int e = c.bt_ptr[k]; e < c.bt_ptr[k + 1]; ++e) t += c.kv[c.bt_q[e]] * xv[c.bt_var[e]];
          t -= c.dq[k];
          if (t > P.eps_abs) viol++;
          if (t > best) {
            best = t;
            bi = k;
          }
        }
        viol = block_sum_int(viol, redi);
        block_select(best, bi, true, red, redi);
        if (viol == 0) {
          converged = 1;
          break;
        }
        if (bi < 0) {
          converged = 0;
          break;
        }
        nxt_active = bi;
        // update_rhs (src/nasoq.cpp:880-889): the constraint's row as the rhs
        for (int i = tid; i < N; i += nt) c.rhs[i] = 0.0;
        __syncthreads();
        for (int e = c.bt_ptr[nxt_active] + tid; e < c.bt_ptr[nxt_active + 1]; e += nt)
          c.rhs[c.bt_var[e]] = c.kv[c.bt_q[e]];
        __syncthreads();
        BQ_T1(c, PH_SELECT);
      }
      // solve_kkt (src/nasoq.cpp:918-957)
      if (typ == 1) {
        BQ_T0(c);
        sort_mlist(c);
        factor_marked(c);
        build_vlist(c);
        typ = 0;
        BQ_T1(c, PH_FACTOR);
      }
      {
        BQ_T0(c);
        precond(c, c.rhs, c.sol);
        solves++;
        steps += refine(c, c.rhs, c.sol, P.outer, P.inner, flexible, adaptive, a.refine_tol, P.tol_abs, P.tol_rel, gs);
        BQ_T1(c, PH_REFINE);
      }
      const long long tu0 = clock64();
      // step lengths (src/nasoq.cpp:852-878)
      double dual_step = DMAX;
      int drop = -1;
      for (int t = tid; t < nact; t += nt) {
        const int k = c.alist[t];
        const double lm = c.sol[c.base + k];
        if (lm > 0.0) {
          const double ratio = zv[k] / lm;
          if (drop < 0 || ratio < dual_step || (ratio == dual_step && k < drop)) {
            dual_step = ratio;
            drop = k;
          }
        }
      }
      block_select(dual_step, drop, false, red, redi);
      if (drop < 0) dual_step = DMAX;
      if (tid == 0) {
        double bdotx = 0.0, ddotb = 0.0;
        for (int e = c.bt_ptr[nxt_active]; e < c.bt_ptr[nxt_active + 1]; ++e) {
          bdotx += c.kv[c.bt_q[e]] * xv[c.bt_var[e]];
          ddotb += c.kv[c.bt_q[e]] * c.sol[c.bt_var[e]];
        }
        double prime_step = DMAX;
        if (!(ddotb < P.zero_thresh)) prime_step = -(c.dq[nxt_active] - bdotx) / ddotb;
        s_dbl[0] = prime_step;
      }
      __syncthreads();
      const double prime_step = s_dbl[0];
      if (drop >= 0) nxt_drop = drop;
      const double step = prime_step > dual_step ? dual_step : prime_step;
      if (step == DMAX) {
        converged = 0;
        break;
      }
      const bool dual_only = prime_step == DMAX && step == dual_step;
      // update_primal / update_dual (src/nasoq.cpp:612-632)
      if (!dual_only)
        for (int i = tid; i < n; i += nt) xv[i] = xv[i] - step * c.sol[i];
      for (int i = tid; i < meq; i += nt) yv[i] -= step * c.sol[n + i];
      for (int t = tid; t < nact; t += nt) {
        const int k = c.alist[t];
        zv[k] -= step * c.sol[c.base + k];
      }
      __syncthreads();
      if (tid == 0) {
        zv[nxt_active] = zv[nxt_active] + step;
        int add = -1, del = -1;
        if (dual_only) del = nxt_drop;
        else if (step == prime_step) add = nxt_active;
        else if (step == dual_step) del = nxt_drop;
        if (add >= 0) {
          const bool fresh = !c.act[add];
          edit_constraint(c, add, true);
          if (fresh && nact < mineq) c.alist[nact++] = add;
          s_int[1] = 1;
        } else if (del >= 0) {
          edit_constraint(c, del, false);
          int pos = -1;
          for (int t = 0; t < nact; ++t)
            if (c.alist[t] == del) pos = t;
          if (pos >= 0) {
            for (int t = pos; t + 1 < nact; ++t) c.alist[t] = c.alist[t + 1];
            nact--;
          }
          s_int[1] = 0;
        } else {
          s_int[1] = -1;
        }
        s_int[0] = nact;
      }
      __syncthreads();
      nact = s_int[0];
      if (s_int[1] >= 0) {
        to_add = s_int[1];
        typ = 1;
      }
      num_iter++;
      if (c.cyc && tid == 0) {
        c.cyc[PH_UPDATE] += (unsigned long long)(clock64() - tu0);
        c.cyc[PH_ITER] += 1;
      }
    }
    // Polish (adaptive refinement only): the updates x -= step * descent
    // carry each solve's residual (1e-12 relative) through every iteration,
    // so the final point is recomputed as the equality-constrained solution
    // on the final active set (constraints whose multipliers come out
    // negative are dropped and the solve repeated); if the point then
    // violates a constraint, the active-set iteration continues from it (at
    // most twice).  The reference's fixed schedule runs to 1e-15 and needs
    // none of this.
    if (!adaptive || !converged || pol >= 2) break;
    // no iteration since the initial solution: it already is the solution on
    // the final active set (negative multipliers were dropped before), so
    // polishing would repeat the same solve
    if (pol == 0 && num_iter == 0) break;
    // the final solution is refined further than the loop's solves: after a
    // long trajectory its active set is settled, and its KKT norms decide the
    // status
    const double polish_tol = fmin(a.refine_tol, 1e-12);
    if (*c.nmark > 0) {
      sort_mlist(c);
      factor_marked(c);
      build_vlist(c);
    }
    typ = 0;
    for (int i = tid; i < N; i += nt) {
      double v = 0.0;
      if (i < n) v = -c.q[i];
      else if (i < c.base) v = c.bq[i - n];
      else if (c.act[i - c.base]) v = c.dq[i - c.base];
      c.rhs[i] = v;
    }
    __syncthreads();
    precond(c, c.rhs, c.sol);
    solves++;
    steps += refine(c, c.rhs, c.sol, P.outer, P.inner, flexible, adaptive, polish_tol, P.tol_abs, P.tol_rel, gs);
    // a negative multiplier: that constraint does not belong to the active
    // set of this point; drop it and solve again (at most three times)
    for (int rep = 0; rep < 3; ++rep) {
      if (tid == 0) {
        int nd = 0;
        for (int t = 0; t < nact;) {
          const int k = c.alist[t];
          if (c.sol[c.base + k] < 0.0) {
            edit_constraint(c, k, false);
            for (int u = t; u + 1 < nact; ++u) c.alist[u] = c.alist[u + 1];
            nact--;
            nd++;
          } else {
            ++t;
          }
        }
        s_int[0] = nact;
        s_int[2] = nd;
      }
      __syncthreads();
      nact = s_int[0];
      if (s_int[2] == 0) break;
      sort_mlist(c);
      factor_marked(c);
      build_vlist(c);
      for (int i = c.base + tid; i < N; i += nt)
        if (!c.act[i - c.base]) c.rhs[i] = 0.0;
      __syncthreads();
      precond(c, c.rhs, c.sol);
      solves++;
      steps += refine(c, c.rhs, c.sol, P.outer, P.inner, flexible, adaptive, polish_tol, P.tol_abs, P.tol_rel, gs);
    }
    for (int k = tid; k < mineq; k += nt)
      if (!c.act[k]) zv[k] = 0.0;
    for (int i = tid; i < n; i += nt) xv[i] = c.sol[i];
    for (int i = tid; i < meq; i += nt) yv[i] = c.sol[n + i];
    for (int t = tid; t < nact; t += nt) {
      const int k = c.alist[t];
      zv[k] = c.sol[c.base + k];
    }
    __syncthreads();
    int viol = 0;
    for (int k = tid; k < mineq; k += nt) {
      double t = 0.0;
      for (int e = c.bt_ptr[k]; e < c.bt_ptr[k + 1]; ++e) t += c.kv[c.bt_q[e]] * xv[c.bt_var[e]];
      if (t - c.dq[k] > P.eps_abs) viol++;
    }
    viol = block_sum_int(viol, redi);
    if (viol == 0) break;
    converged = 0;
    to_add = 1;
    }

    // ---- results: objective and KKT norms (src/nasoq.cpp:712-728, 1013-1106)
    // Hx, Ax, Cx and H x + A^T y + C^T z from the original values
    for (int i = tid; i < N; i += nt) {
      double v = 0.0;
      if (i < n) v = xv[i];
      c.w[i] = v;
      double u = v;
      if (i >= n && i < c.base) u = yv[i - n];
      else if (i >= c.base) u = zv[i - c.base];
      c.tmp[i] = u;
    }
    __syncthreads();
    double quad = 0.0, lin = 0.0, lag = 0.0;
    for (int i = tid; i < n; i += nt) {
      double hx = 0.0, full = 0.0;
      for (int qq = c.Rp[i]; qq < c.Rp[i + 1]; ++qq) {
        const int j = c.Rj[qq];
        const double v = c.kv[c.Rq[qq]];
        if (j < n) hx += v * c.w[j];
        full += v * c.tmp[j];
      }
      quad += hx * xv[i];
      lin += c.q[i] * xv[i];
      lag = fmax(lag, fabs(full + c.q[i]));
    }
    double cons = 0.0, dual_obj = 0.0, nonneg = 0.0, comp = 0.0;
    for (int k = tid; k < mineq; k += nt) {
      double t = 0.0;
      for (int e = c.bt_ptr[k]; e < c.bt_ptr[k + 1]; ++e) t += c.kv[c.bt_q[e]] * xv[c.bt_var[e]];
      t -= c.dq[k];
      cons = fmax(cons, t < 0.0 ? 0.0 : t);
      dual_obj += t * zv[k];
      nonneg = fmax(nonneg, zv[k] > 0.0 ? 0.0 : fabs(zv[k]));
      comp = fmax(comp, fabs(zv[k] * t));
    }
    for (int r = tid; r < meq; r += nt) {
      double t = 0.0;
      for (int e = c.eq_ptr[r]; e < c.eq_ptr[r + 1]; ++e) t += c.kv[c.eq_q[e]] * xv[c.eq_var[e]];
      cons = fmax(cons, fabs(t - c.bq[r]));
    }
    // a non-finite solution (non-finite data, or a breakdown the loop could
    // not recover from) is never reported as converged
    int nonfin = 0;
    for (int i = tid; i < N; i += nt)
      if (!isfinite(c.tmp[i]) || !isfinite(c.w[i])) nonfin = 1;
    nonfin = block_sum_int(nonfin, redi);
    quad = block_sum(quad, red);
    lin = block_sum(lin, red);
    dual_obj = block_sum(dual_obj, red);
    double mx[4] = {lag, cons, nonneg, comp};
    for (int m = 0; m < 4; ++m) {
      double v = mx[m];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
      __syncthreads();
      if (lane_id() == 0) red[warp_id()] = v;
      __syncthreads();
      if (tid == 0) {
        double w = 0.0;
        for (int t = 0; t < num_warps(); ++t) w = fmax(w, red[t]);
        s_dbl[m] = w;
      }
      __syncthreads();
      mx[m] = s_dbl[m];
      __syncthreads();
    }
    for (int t = tid; t < mineq; t += nt) as_out[t] = t < nact ? c.alist[t] : -1;
    if (tid == 0) {
      BResult &R = a.res[pi];
      R.num_iter = num_iter;
      R.active_size = nact;
      R.flags = s_status | (nonfin ? ST_NONFINITE : 0);
      R.refine_steps = steps;
      R.solves = solves;
      R.warm_dropped = warm_dropped;
      R.primal_obj = 0.5 * quad + lin;
      R.dual_obj = dual_obj;
      R.objective = R.primal_obj + dual_obj;
      R.lag_res = mx[0];
      R.cons_sat_norm = mx[1];
      R.non_negativity_infn = mx[2];
      R.complementarity_infn = mx[3];
      int st;
      if (nonfin) st = 3;      // NotConverged
      else if (!converged) st = 0;  // check_solve_status: Infeasible when the loop did not converge
      else if (mx[0] <= P.eps_abs && mx[1] <= P.eps_abs && mx[2] <= P.eps_abs) st = 1;
      else if (mx[1] <= P.eps_abs) st = 2;
      else st = 3;
      R.status = st;
      if (c.cyc) c.cyc[PH_TOTAL] += (unsigned long long)(clock64() - tp0);
    }
    __syncthreads();
  }
  if (a.prof && tid < PH_N) atomicAdd(a.prof + tid, s_cyc[tid]);
}

// batch_fp64.cu compiles this file again with NQG_BATCH_FP64_UNIT defined for
// the FP64 instantiation alone (the two instantiations then build in
// parallel); the non-template kernels and host functions belong to this unit.
#ifndef NQG_BATCH_FP64_UNIT

// Warm-start sets from per-constraint scores (e.g. the logits of the active-set
// model): problem i proposes every constraint k with scores[i * ld + k] >
// threshold, in ascending order, except one parallel to a constraint it
// already proposed (same variables, proportional coefficients -- the two
// sides of a box): both active would make the KKT matrix singular.  A
// problem with no proposal keeps a cold start.  One warp per problem: lanes
// read 32 scores at a time (coalesced); the candidates of a chunk are taken
// in constraint order, each checked by all lanes at once against the
// constraints already proposed.
__global__ void k_ws_scores(int nprob, BProb *probs, const BPat *pats, const int *ipool, const double *dpool,
                            int *iout, const float *scores, int ld, float thr) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= nprob) return;
  BProb &P = probs[i];
  const BPat &pt = pats[P.pat];
  const int *bt_ptr = ipool + pt.o_bt_ptr, *bt_var = ipool + pt.o_bt_var, *bt_q = ipool + pt.o_bt_q;
  const double *kv = dpool + P.o_kv;
  int *as = iout + P.o_as;
  const float *sc = scores + (size_t)i * ld;
  int cnt = 0;
  const int mi = min(pt.mineq, ld);
  for (int c0 = 0; c0 < mi; c0 += 32) {
    const int kk = c0 + lane;
    unsigned cand = __ballot_sync(0xffffffffu, kk < mi && sc[kk] > thr);
    while (cand) {
      const int k = c0 + __ffs(cand) - 1;
      cand &= cand - 1;
      const int ka = bt_ptr[k], kn = bt_ptr[k + 1] - ka;
      bool parallel = false;
      for (int t = lane; t < cnt; t += 32) {
        const int j = as[t], ja = bt_ptr[j], jn = bt_ptr[j + 1] - ja;
        if (jn != kn || kn == 0) continue;
        bool same = true;
        const double r = kv[bt_q[ka]] / kv[bt_q[ja]];
        for (int e = 0; e < kn && same; ++e)
          same = bt_var[ka + e] == bt_var[ja + e] &&
                 fabs(kv[bt_q[ka + e]] - r * kv[bt_q[ja + e]]) <= 1e-12 * fabs(kv[bt_q[ka + e]]);
        parallel = parallel || same;
      }
      if (!__any_sync(0xffffffffu, parallel)) {
        if (lane == 0) as[cnt] = k;
        ++cnt;
        __syncwarp();
      }
    }
  }
  if (lane == 0) P.ws_n = cnt > 0 ? cnt : -1;
}

// One block per problem: its q, b and d from the stacked staging buffer.
__global__ void k_scatter_vectors(int nprob, const BProb *probs, const BPat *pats, const int64_t *voff,
                                  const double *stage, double *dpool) {
  const int i = blockIdx.x;
  if (i >= nprob) return;
  const BProb &P = probs[i];
  const BPat &pt = pats[P.pat];
  const int64_t oq = voff[3 * i], ob = voff[3 * i + 1], od = voff[3 * i + 2];
  if (oq >= 0)
    for (int t = threadIdx.x; t < pt.n; t += blockDim.x) dpool[P.o_q + t] = stage[oq + t];
  if (ob >= 0)
    for (int t = threadIdx.x; t < pt.meq; t += blockDim.x) dpool[P.o_b + t] = stage[ob + t];
  if (od >= 0)
    for (int t = threadIdx.x; t < pt.mineq; t += blockDim.x) dpool[P.o_d + t] = stage[od + t];
}

int batch_scatter_vectors(int nprob, const BProb *probs, const BPat *pats, const int64_t *voff, const double *stage,
                          double *dpool, cudaStream_t st) {
  if (nprob <= 0) return NQG_OK;
  k_scatter_vectors<<<nprob, 128, 0, st>>>(nprob, probs, pats, voff, stage, dpool);
  return cudaGetLastError() == cudaSuccess ? NQG_OK : NQG_ERR_CUDA;
}

__global__ void k_ws_clear(int nprob, BProb *probs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nprob) probs[i].ws_n = -1;
}

int batch_ws_from_scores(int nprob, BProb *probs, const BPat *pats, const int *ipool, const double *dpool, int *iout,
                         const float *scores, int ld, float thr, cudaStream_t st) {
  k_ws_scores<<<(nprob + 7) / 8, 256, 0, st>>>(nprob, probs, pats, ipool, dpool, iout, scores, ld, thr);
  return cudaGetLastError() == cudaSuccess ? NQG_OK : NQG_ERR_CUDA;
}

int batch_ws_clear(int nprob, BProb *probs, cudaStream_t st) {
  k_ws_clear<<<(nprob + 127) / 128, 128, 0, st>>>(nprob, probs);
  return cudaGetLastError() == cudaSuccess ? NQG_OK : NQG_ERR_CUDA;
}

size_t batch_smem_bytes(const BArgs &a, size_t tsize) {
  auto up = [](size_t b) { return (b + 15) / 16 * 16; };
  size_t wf = 0;
  if (a.warp_factor) {
    const size_t wcap = (size_t)std::min(a.w_max, 32), rcap = (size_t)std::min(a.nr_max, 32);
    wf = up(WF_WARPS * wcap * rcap * tsize) + 2 * up(WF_WARPS * wcap * tsize) + up(WF_WARPS * wcap * sizeof(int)) +
         up((size_t)WF_WARPS * 64 * tsize);
  }
  return up((size_t)a.N_max * sizeof(int)) + up((size_t)a.N_max * tsize) + up((size_t)a.nr_max * a.w_max * tsize) +
         up((size_t)a.w_max * 32 * tsize) + 2 * up((size_t)a.w_max * tsize) + up((size_t)a.w_max * sizeof(int)) +
         up((size_t)a.w_max * a.w_max * tsize) + 4 * up((size_t)(a.nlev_max + 1) * sizeof(int)) + up((size_t)a.ns_max) +
         up((size_t)a.mi_max) + wf + (size_t)a.stage_bytes;
}

#endif  // NQG_BATCH_FP64_UNIT

// Raises the kernel's dynamic shared-memory limit to smem_attr (outside any
// stream capture) and returns how many CTAs of `smem` bytes fit on an SM.
template <class T> int batch_prepare(int threads, size_t smem_attr, size_t smem, int *blocks_per_sm) {
  if (cudaFuncSetAttribute(k_nasoq_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_attr) !=
      cudaSuccess)
    return NQG_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_nasoq_batch<T>, threads, smem) != cudaSuccess)
    return NQG_ERR_CUDA;
  return NQG_OK;
}

template <class T> int launch_batch(const BArgs &a, int grid, int threads, size_t smem, cudaStream_t st) {
  k_nasoq_batch<T><<<grid, threads, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? NQG_OK : NQG_ERR_CUDA;
}

#ifdef NQG_BATCH_FP64_UNIT
template int launch_batch<double>(const BArgs &, int, int, size_t, cudaStream_t);
template int batch_prepare<double>(int, size_t, size_t, int *);
#else
template int launch_batch<float>(const BArgs &, int, int, size_t, cudaStream_t);
template int batch_prepare<float>(int, size_t, size_t, int *);
#endif

}  // namespace nqg
