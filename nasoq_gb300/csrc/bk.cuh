// Bunch-Kaufman building blocks shared by the level-scheduled factorization
// (numeric.cu) and the batched QP solver (batch.cu): block-wide argmax, the
// Bunch-Kaufman factorization of one supernode diagonal block
// (LAPACK dsytrf('L') pivot rule, alpha = (1+sqrt(17))/8) with explicit
// interchanges, and the solve of the rows below the block.  All functions are
// CTA-scope: every thread of the block calls them.
#pragma once
#include <cuda_runtime.h>

#include "plan.hpp"

namespace nqg {
namespace {

constexpr int BK_SMALL = 64;  // diagonal blocks up to this width live in shared memory

__device__ __forceinline__ void flag_status(int *st, int bits) { atomicOr(st, bits); }

template <class T> __device__ __forceinline__ T tabs(T v) { return v < T(0) ? -v : v; }

// Block-wide argmax of |value| with the smallest index winning ties (the
// LAPACK idamax convention).  Every thread passes its candidate; returns the
// winner to all threads.  `sv`/`si` are shared scratch of blockDim/32 entries.
template <class T>
__device__ void block_argmax(T &v, int &idx, T *sv, int *si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T ov = __shfl_down_sync(0xffffffffu, v, o);
    int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (oi >= 0 && (idx < 0 || ov > v || (ov == v && oi < idx))) {
      v = ov;
      idx = oi;
    }
  }
  __syncthreads();
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = idx;
  }
  __syncthreads();
  if (wid == 0) {
    v = lane < nw ? sv[lane] : T(-1);
    idx = lane < nw ? si[lane] : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, v, o);
      int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (oi >= 0 && (idx < 0 || ov > v || (ov == v && oi < idx))) {
        v = ov;
        idx = oi;
      }
    }
    if (lane == 0) {
      sv[0] = v;
      si[0] = idx;
    }
  }
  __syncthreads();
  v = sv[0];
  idx = si[0];
  __syncthreads();
}

// Bunch-Kaufman (alpha = (1+sqrt(17))/8) on the w-by-w lower-stored block
// `a` (column-major, leading dimension lda), leaving L in explicit form
// (P A P^T = L D L^T): every interchange also swaps the two rows in all
// previously computed columns.  On return a holds L with unit diagonal and
// zeroed 2x2 sub-diagonals; D/E get the diagonal and 2x2 sub-diagonals;
// perm[m] = original local column now at position m.
// Largest diagonal block k_bk_global stages in shared memory (bytes).
constexpr size_t BKG_STAGE_MAX = 200 * 1024;

template <class T>
__device__ void bk_factor(T *a, int lda, int w, T *D, T *E, int *perm, int *status, bool *pivoted_out) {
  __shared__ T red_v[32];
  __shared__ int red_i[32];
  __shared__ int s_kp, s_kstep, s_zero;
  __shared__ T s_wk[BK_SMALL * 2];
  const T alpha = (T)((1.0 + sqrt(17.0)) / 8.0);
  const int tid = threadIdx.x, nt = blockDim.x;
  bool pivoted = false;
  for (int m = tid; m < w; m += nt) perm[m] = m;
  __syncthreads();
  int k = 0;
  while (k < w) {
    // ---- pivot search on column k
    T absakk = tabs(a[k + (size_t)k * lda]);
    T cv = T(-1);
    int ci = -1;
    for (int i = k + 1 + tid; i < w; i += nt) {
      T v = tabs(a[i + (size_t)k * lda]);
      if (ci < 0 || v > cv) {
        cv = v;
        ci = i;
      }
    }
    block_argmax(cv, ci, red_v, red_i);
    T colmax = ci >= 0 ? cv : T(0);
    int imax = ci;
    int kp = k, kstep = 1, zero = 0;
    if ((absakk >= colmax ? absakk : colmax) == T(0) || absakk != absakk) {
      zero = 1;
    } else if (absakk >= alpha * colmax) {
      kp = k;
    } else {
      // rowmax: off-diagonal max of row/column imax inside the trailing block
      T rv = T(-1);
      int ri = -1;
      for (int j = k + tid; j < w; j += nt) {
        if (j == imax) continue;
        T v = j < imax ? tabs(a[imax + (size_t)j * lda]) : tabs(a[j + (size_t)imax * lda]);
        if (ri < 0 || v > rv) {
          rv = v;
          ri = j;
        }
      }
      block_argmax(rv, ri, red_v, red_i);
      T rowmax = rv;
      if (absakk >= alpha * colmax * (colmax / rowmax)) {
        kp = k;
      } else if (tabs(a[imax + (size_t)imax * lda]) >= alpha * rowmax) {
        kp = imax;
      } else {
        kp = imax;
        kstep = 2;
      }
    }
    if (tid == 0) {
      s_kp = kp;
      s_kstep = kstep;
      s_zero = zero;
    }
    __syncthreads();
    kp = s_kp;
    kstep = s_kstep;
    zero = s_zero;
    const int kk = k + kstep - 1;
    // a NaN pivot is reported by the non-finite check, not as a zero pivot
    if (zero && tid == 0 && absakk == absakk) flag_status(status, ST_ZERO_PIVOT);
    // ---- symmetric interchange of kk and kp (kp > kk)
    if (kp != kk) {
      pivoted = true;
      for (int i = kp + 1 + tid; i < w; i += nt) {
        T t = a[i + (size_t)kk * lda];
        a[i + (size_t)kk * lda] = a[i + (size_t)kp * lda];
        a[i + (size_t)kp * lda] = t;
      }
      for (int j = kk + 1 + tid; j < kp; j += nt) {
        T t = a[j + (size_t)kk * lda];
        a[j + (size_t)kk * lda] = a[kp + (size_t)j * lda];
        a[kp + (size_t)j * lda] = t;
      }
      // rows kk and kp of the columns to the left of the current pivot
      // (for a 2x2 pivot this includes column k: LAPACK swaps A(k+1,k), A(kp,k))
      const int ncols_left = kstep == 2 ? k + 1 : k;
      for (int c = tid; c < ncols_left; c += nt) {
        T t = a[kk + (size_t)c * lda];
        a[kk + (size_t)c * lda] = a[kp + (size_t)c * lda];
        a[kp + (size_t)c * lda] = t;
      }
      if (tid == 0) {
        T t = a[kk + (size_t)kk * lda];
        a[kk + (size_t)kk * lda] = a[kp + (size_t)kp * lda];
        a[kp + (size_t)kp * lda] = t;
        int pt = perm[kk];
        perm[kk] = perm[kp];
        perm[kp] = pt;
      }
    }
    __syncthreads();
    // ---- elimination
    if (kstep == 1) {
      if (!zero) {
        const T r1 = T(1) / a[k + (size_t)k * lda];
        const int m = w - k - 1;
        // trailing rank-1 update of the lower triangle, then scale the column
        for (int e = tid; e < m * m; e += nt) {
          int jj = e / m, ii = e % m;
          if (ii < jj) continue;
          int i = k + 1 + ii, j = k + 1 + jj;
          a[i + (size_t)j * lda] -= r1 * a[j + (size_t)k * lda] * a[i + (size_t)k * lda];
        }
        __syncthreads();
        for (int i = k + 1 + tid; i < w; i += nt) a[i + (size_t)k * lda] *= r1;
      }
      if (tid == 0) {
        D[k] = a[k + (size_t)k * lda];
        E[k] = T(0);
      }
    } else {
      // 2x2 pivot on rows/cols k, k+1
      T d21 = a[k + 1 + (size_t)k * lda];
      T d11 = a[k + 1 + (size_t)(k + 1) * lda] / d21;
      T d22 = a[k + (size_t)k * lda] / d21;
      T t = T(1) / (d11 * d22 - T(1));
      d21 = t / d21;
      const int m = w - k - 2;
      // multipliers for all trailing rows j (kept in shared or recomputed)
      for (int base = 0; base < m; base += BK_SMALL) {
        const int cnt = min(BK_SMALL, m - base);
        for (int q = tid; q < cnt; q += nt) {
          int j = k + 2 + base + q;
          T ajk = a[j + (size_t)k * lda], ajk1 = a[j + (size_t)(k + 1) * lda];
          s_wk[2 * q] = d21 * (d11 * ajk - ajk1);
          s_wk[2 * q + 1] = d21 * (d22 * ajk1 - ajk);
        }
        __syncthreads();
        // update columns j in [base, base+cnt): a(i,j) -= a(i,k) wk_j + a(i,k+1) wkp1_j, i >= j
        for (int e = tid; e < cnt * m; e += nt) {
          int q = e / m, ii = e % m;
          int j = k + 2 + base + q, i = k + 2 + ii;
          if (i < j) continue;
          a[i + (size_t)j * lda] -= a[i + (size_t)k * lda] * s_wk[2 * q] + a[i + (size_t)(k + 1) * lda] * s_wk[2 * q + 1];
        }
        __syncthreads();
        // multipliers of rows whose trailing updates are all done can be written:
        // columns k, k+1 are read by later chunks (rows i >= j), so stage them.
        for (int q = tid; q < cnt; q += nt) {
          int j = k + 2 + base + q;
          // keep the multiplier in the upper triangle slot (unused) temporarily
          a[k + (size_t)j * lda] = s_wk[2 * q];
          a[k + 1 + (size_t)j * lda] = s_wk[2 * q + 1];
        }
        __syncthreads();
      }
      for (int j = k + 2 + tid; j < w; j += nt) {
        a[j + (size_t)k * lda] = a[k + (size_t)j * lda];
        a[j + (size_t)(k + 1) * lda] = a[k + 1 + (size_t)j * lda];
        a[k + (size_t)j * lda] = T(0);
        a[k + 1 + (size_t)j * lda] = T(0);
      }
      if (tid == 0) {
        D[k] = a[k + (size_t)k * lda];
        D[k + 1] = a[k + 1 + (size_t)(k + 1) * lda];
        E[k] = a[k + 1 + (size_t)k * lda];
        E[k + 1] = T(0);
        a[k + 1 + (size_t)k * lda] = T(0);
      }
    }
    __syncthreads();
    k += kstep;
  }
  for (int m = tid; m < w; m += nt) a[m + (size_t)m * lda] = T(1);
  __syncthreads();
  if (pivoted_out) *pivoted_out = pivoted;
}

// Block-wide OR of a per-thread flag.
__device__ bool block_any(bool f) { return __syncthreads_or(f ? 1 : 0) != 0; }

// Panel rows [w, nrow): columns permuted by perm, solved with the unit lower
// L11^T and scaled by D^-1 (1x1: times 1/d; 2x2: Cramer's rule with
// 1/det, the arithmetic of blocked_2by2_solver).  One thread per row.
template <class T>
__device__ void panel_solve_rows(T *Ls, int nrow, int w, const T *l11, int ld11, const T *D, const T *E,
                                 const int *perm, T *rowbuf, int rb_ld, bool permute) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int r0 = w; r0 < nrow; r0 += nt) {
    const int r = r0 + tid;
    const bool act = r < nrow;
    if (act) {
      for (int j = 0; j < w; ++j) {
        int src = permute ? perm[j] : j;
        rowbuf[j * rb_ld + tid] = Ls[r + (size_t)src * nrow];
      }
      for (int j = 0; j < w; ++j) {
        T x = rowbuf[j * rb_ld + tid];
        for (int t = 0; t < j; ++t) x -= rowbuf[t * rb_ld + tid] * l11[j + (size_t)t * ld11];
        rowbuf[j * rb_ld + tid] = x;
      }
      for (int j = 0; j < w; ++j) {
        if (E[j] == T(0)) {
          T inv = T(1) / D[j];
          Ls[r + (size_t)j * nrow] = rowbuf[j * rb_ld + tid] * inv;
        } else {
          T s = E[j];
          T det = D[j] * D[j + 1] - s * s;
          T inv = T(1) / det;
          T x1 = rowbuf[j * rb_ld + tid], x2 = rowbuf[(j + 1) * rb_ld + tid];
          Ls[r + (size_t)j * nrow] = (x1 * D[j + 1] - x2 * s) * inv;
          Ls[r + (size_t)(j + 1) * nrow] = (x2 * D[j] - x1 * s) * inv;
          ++j;
        }
      }
    }
  }
}


}  // namespace
}  // namespace nqg
