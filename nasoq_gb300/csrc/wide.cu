// Blocked Bunch-Kaufman factorization of one wide supernode (all nrow x w
// values of the supernode at once), for diagonal blocks too wide for a single
// CTA.
//
// The pivot search is restricted to the w x w diagonal block, exactly as
// LAPACK dsytrf('L') on that block in the reference
// (src/ldl/Serial_blocked_ldl_02_2.cpp:130); the rows below the block are
// carried through every interchange (as columns) and every update, which
// yields the reference's dlapmt + dtrsm + blocked_2by2_solver panel result
// (:137-161) without a separate triangular solve.
//
// Per panel of nb columns (left-looking inside the panel, the dlasyf scheme):
//   k_wide_panel    cooperative launch, G CTAs, rows grid-strided; one grid
//                   barrier per column when no interchange is needed, three
//                   when one is.  W holds the updated panel columns (= L D).
//   k_wide_trailing A22 -= L21 W21^T over the remaining columns (lower
//                   trapezoid incl. all rows below the block), 2-D tiles.
// Every spin-wait is bounded: on timeout the kernel records ST_TIMEOUT and
// all CTAs leave through the same poisoned barrier.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <type_traits>

#include "coop.cuh"
#include "plan.hpp"
#include "tcgen05.cuh"
#include "tf32x3.cuh"

namespace nqg {

namespace {

// Packed operands of the tcgen05 updates: blocks of 128 rows x one chunk of K,
// swizzled K-major, hi part then lo part.  A chunk is 128 bytes of a row:
// 64 K entries of split BF16 (the default), or 32 of split TF32
// (NASOQ_GB300_SPLIT=tf32: twice the operand bytes and MMA steps per
// product, 2^-22 instead of 2^-16 relative representation error).
__host__ __device__ constexpr int pk_chunk(bool bf) { return bf ? 64 : 32; }
bool pk_bf16() {
  const char *e = std::getenv("NASOQ_GB300_SPLIT");
  return !(e && std::string(e) == "tf32");
}

// One 16-byte unit of a packed row: 4 K entries (TF32) or 8 (BF16, two per
// word, lower K in the low half), split into hi / lo, at unit position
// c ^ (r % 8) of row r of the hi and lo blocks.
template <bool BF>
__device__ __forceinline__ void pk_store_unit(unsigned char *hi, unsigned char *lo, int r, int c, const float *x) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if constexpr (BF) {
      t5::bf16_split2(x[2 * q], x[2 * q + 1], h[q], l[q]);
    } else {
      h[q] = t5::tf32_rna(x[q]);
      l[q] = t5::tf32_rna(x[q] - __uint_as_float(h[q]));
    }
  }
  const int off = r * 128 + ((c ^ (r & 7)) << 4);
  *reinterpret_cast<uint4 *>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4 *>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

constexpr int WP_THREADS = 256;
constexpr int WP_NB = 64;  // widest panel; the row cache holds WP_NB + 2 columns

template <class T> __device__ __forceinline__ T tabs_w(T v) { return v < T(0) ? -v : v; }

// Block-local argmax (value, smallest index on ties) of the thread
// candidates; result valid in thread 0.
template <class T> __device__ void cta_argmax(T &v, int &i) {
  __shared__ T sv[32];
  __shared__ int si[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T ov = __shfl_down_sync(0xffffffffu, v, o);
    int oi = __shfl_down_sync(0xffffffffu, i, o);
    if (oi >= 0 && (i < 0 || ov > v || (ov == v && oi < i))) {
      v = ov;
      i = oi;
    }
  }
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = i;
  }
  __syncthreads();
  if (wid == 0) {
    v = lane < nw ? sv[lane] : T(-1);
    i = lane < nw ? si[lane] : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, v, o);
      int oi = __shfl_down_sync(0xffffffffu, i, o);
      if (oi >= 0 && (i < 0 || ov > v || (ov == v && oi < i))) {
        v = ov;
        i = oi;
      }
    }
  }
  __syncthreads();
}

// Reduce the G partial (value, index) pairs of one phase; every CTA does this
// redundantly so that all take the same pivoting decision.
template <class T> __device__ void reduce_partials(const double *pv, const int *pi, int G, T &v, int &idx) {
  __shared__ double rv;
  __shared__ int ri;
  if (threadIdx.x < 32) {
    double bv = -1.0;
    int bi = -1;
    for (int g = threadIdx.x; g < G; g += 32) {
      double x = __ldcg(pv + g);
      int xi = __ldcg(pi + g);
      if (xi >= 0 && (bi < 0 || x > bv || (x == bv && xi < bi))) {
        bv = x;
        bi = xi;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, bv, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) {
        bv = ov;
        bi = oi;
      }
    }
    if (threadIdx.x == 0) {
      rv = bv;
      ri = bi;
    }
  }
  __syncthreads();
  v = (T)rv;
  idx = ri;
  __syncthreads();
}

// Panel exchange: every CTA publishes one 64-bit word per synchronisation,
// (candidate << 8) | epoch, into its own slot of the current parity; one warp
// of every CTA then polls all slots until each carries this epoch and takes
// their maximum.  This is the grid barrier and the pivot search in one step,
// without atomics.  The slot is written after __syncthreads + __threadfence
// (the CTA's earlier writes are ordered before it) and read back before a
// __threadfence (later reads see the other CTAs' writes); data written by
// other CTAs is read with ld.cg.  Two parities let a fast CTA publish the
// next exchange while a slow one still reads this one.  The wait is bounded.
__device__ bool grid_exchange(WideCtl *ctl, unsigned &epoch, unsigned long long cand, int *status,
                              unsigned long long &best) {
  __shared__ unsigned long long s_best;
  __shared__ int s_ok;
  ++epoch;
  const unsigned e = epoch & 0xFFu;  // at most 255 exchanges per panel launch: never 0
  const int par = epoch & 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    *(volatile unsigned long long *)&ctl->pslot[par][blockIdx.x] = (cand << 8) | e;
  }
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    long long it = 0;
    const long long lim_ = wait_limit(ctl);
    int ok = 1;
    unsigned long long m = 0;
    while (true) {
      bool all = true;
      m = 0;
      for (int g = lane; g < (int)gridDim.x; g += 32) {
        const unsigned long long v = *(volatile unsigned long long *)&ctl->pslot[par][g];
        if ((unsigned)(v & 0xFFu) != e) all = false;
        else m = max(m, v >> 8);
      }
      if (__all_sync(0xffffffffu, all)) break;
      int ab = lane == 0 ? *(volatile int *)&ctl->abort : 0;
      ab = __shfl_sync(0xffffffffu, ab, 0);
      if (ab) {
        ok = 0;
        break;
      }
      if (++it > lim_) {
        if (lane == 0) {
          atomicOr(status, ST_TIMEOUT);
          atomicExch(&ctl->abort, 1);
        }
        ok = 0;
        break;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __threadfence();
    if (lane == 0) {
      s_best = m;
      s_ok = ok;
    }
  }
  __syncthreads();
  best = s_best;
  return s_ok != 0;
}

// Column-step argmax over the whole grid (valid on return in every thread,
// the same in every CTA).  FP32: the candidate rides in the exchange word as
// (|value| bits << 24) | (0xFFFFFF - row), 0 for none, so the maximum keeps
// the largest value and, among equal values, the smallest row (rows < 2^24).
// FP64: per-CTA partials beside the exchange, reduced redundantly by all.
template <class T>
__device__ bool grid_argmax(T cv, int ci, WideCtl *ctl, int phase, unsigned &epoch, int *status, T &v, int &idx) {
  cta_argmax(cv, ci);
  unsigned long long best = 0;
  if constexpr (sizeof(T) == 4) {
    unsigned long long cand = 0;
    if (ci >= 0) cand = ((unsigned long long)__float_as_uint((float)cv) << 24) | (0xFFFFFFull - (unsigned)ci);
    if (!grid_exchange(ctl, epoch, cand, status, best)) return false;
    if (best == 0ull) {
      v = T(0);
      idx = -1;
    } else {
      v = (T)__uint_as_float((unsigned)(best >> 24));
      idx = 0xFFFFFF - (int)(best & 0xFFFFFFull);
    }
  } else {
    const int par = (epoch + 1) & 1;  // parity of the coming exchange
    double *pv = phase ? ctl->rval[par] : ctl->cval[par];
    int *pi = phase ? ctl->ridx[par] : ctl->cidx[par];
    if (threadIdx.x == 0) {
      pv[blockIdx.x] = (double)cv;
      pi[blockIdx.x] = ci;
    }
    if (!grid_exchange(ctl, epoch, 0ull, status, best)) return false;
    reduce_partials(pv, pi, gridDim.x, v, idx);
  }
  return true;
}

// ---------------------------------------------------------------------------
// FP32 fast panel: the columns of a panel for which Bunch-Kaufman keeps the
// diagonal pivot (|a_cc| >= alpha * colmax, no interchange) -- every column
// once the pivot order has settled.  Every CTA keeps its own copy of the
// panel's diagonal-block rows R = [k0, k0 + nbR): their original entries Sr,
// their W entries Wr and their L entries Lr, computed redundantly with the
// same arithmetic in every CTA.  The pivot W(c, j) and the next update row
// W(c+1, 0..j) are then local, the only value that crosses CTAs is the
// column-max candidate, and the exchange needs no memory fences.  The other
// rows are owned one per thread (512 threads per CTA, L entries cached in
// shared memory).  At the first column that needs a pivot search (or has a
// zero or NaN pivot) every CTA stops with the same decision; kb = columns
// done and ctl->stop tell the host to close this partial panel and hand the
// column to the general kernel.
constexpr int FP_THREADS = 512;

// CTA argmax of packed FP32 candidates (hi = |value| bits, lo = 0xFFFFFF -
// row; 0/0 for none) with redux.sync; result valid in every thread.
__device__ __forceinline__ unsigned long long cta_max_key(unsigned hi, unsigned lo) {
  __shared__ unsigned s_hi[FP_THREADS / 32], s_lo[FP_THREADS / 32];
  __shared__ unsigned long long s_key;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  if (lane == 0) {
    s_hi[wid] = mh;
    s_lo[wid] = ml;
  }
  __syncthreads();
  if (wid == 0) {
    const unsigned h = lane < nw ? s_hi[lane] : 0u, l = lane < nw ? s_lo[lane] : 0u;
    mh = __reduce_max_sync(0xffffffffu, h);
    ml = __reduce_max_sync(0xffffffffu, h == mh ? l : 0u);
    if (lane == 0) s_key = ((unsigned long long)mh << 24) | ml;
  }
  __syncthreads();
  return s_key;
}

// Barrier + maximum over the CTAs' candidate words, without fences (nothing
// else is exchanged).  Same slots, epochs and parities as grid_exchange.
__device__ bool grid_max_nofence(WideCtl *ctl, unsigned &epoch, unsigned long long cand, int *status,
                                 unsigned long long &best) {
  __shared__ unsigned long long s_best;
  __shared__ int s_ok;
  ++epoch;
  const unsigned e = epoch & 0xFFu;
  const int par = epoch & 1;
  if (threadIdx.x == 0) *(volatile unsigned long long *)&ctl->pslot[par][blockIdx.x] = (cand << 8) | e;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    long long it = 0;
    const long long lim_ = wait_limit(ctl);
    int ok = 1;
    unsigned long long m = 0;
    while (true) {
      bool all = true;
      m = 0;
      for (int g = lane; g < (int)gridDim.x; g += 32) {
        const unsigned long long v = *(volatile unsigned long long *)&ctl->pslot[par][g];
        if ((unsigned)(v & 0xFFu) != e) all = false;
        else m = max(m, v >> 8);
      }
      if (__all_sync(0xffffffffu, all)) break;
      int ab = lane == 0 ? *(volatile int *)&ctl->abort : 0;
      ab = __shfl_sync(0xffffffffu, ab, 0);
      if (ab) {
        ok = 0;
        break;
      }
      if (++it > lim_) {
        if (lane == 0) {
          atomicOr(status, ST_TIMEOUT);
          atomicExch(&ctl->abort, 1);
        }
        ok = 0;
        break;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
      s_best = m;
      s_ok = ok;
    }
  }
  __syncthreads();
  best = s_best;
  return s_ok != 0;
}

// Exchange of g <= FP_COLS candidate words per CTA at once (columns j ..
// j+g-1 of a fast panel); best[q] = maximum over the CTAs of word q.
constexpr int FP_COLS = 4;
__device__ bool grid_max_multi(WideCtl *ctl, unsigned &epoch, const unsigned long long (&cand)[FP_COLS], int g,
                               int *status, unsigned long long (&best)[FP_COLS]) {
  __shared__ unsigned long long s_best[FP_COLS];
  __shared__ int s_ok;
  ++epoch;
  const unsigned e = epoch & 0xFFu;
  const int par = epoch & 1;
  const int G = (int)gridDim.x;
  if (threadIdx.x < g) *(volatile unsigned long long *)&ctl->mslot[par][threadIdx.x][blockIdx.x] = (cand[threadIdx.x] << 8) | e;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    long long it = 0;
    const long long lim_ = wait_limit(ctl);
    int ok = 1;
    unsigned long long m[FP_COLS];
    while (true) {
      bool all = true;
#pragma unroll
      for (int q = 0; q < FP_COLS; ++q) {
        m[q] = 0;
        if (q < g)
          for (int b = lane; b < G; b += 32) {
            const unsigned long long v = *(volatile unsigned long long *)&ctl->mslot[par][q][b];
            if ((unsigned)(v & 0xFFu) != e) all = false;
            else m[q] = max(m[q], v >> 8);
          }
      }
      if (__all_sync(0xffffffffu, all)) break;
      int ab = lane == 0 ? *(volatile int *)&ctl->abort : 0;
      ab = __shfl_sync(0xffffffffu, ab, 0);
      if (ab) {
        ok = 0;
        break;
      }
      if (++it > lim_) {
        if (lane == 0) {
          atomicOr(status, ST_TIMEOUT);
          atomicExch(&ctl->abort, 1);
        }
        ok = 0;
        break;
      }
    }
#pragma unroll
    for (int q = 0; q < FP_COLS; ++q) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m[q] = max(m[q], __shfl_xor_sync(0xffffffffu, m[q], o));
      if (lane == 0) s_best[q] = m[q];
    }
    if (lane == 0) s_ok = ok;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < FP_COLS; ++q) best[q] = s_best[q];
  return s_ok != 0;
}

__host__ __device__ constexpr size_t fast_panel_smem(int nb) {
  return ((size_t)nb * FP_THREADS + (size_t)nb * (nb + 1)) * sizeof(float);
}

// Right-looking: after column j, the thread's row and the replicated rows R
// get the rank-1 term L(r, j) W(k0 + j', j) subtracted from every later panel
// column j' at once (independent FMAs), so the next column's W values and
// pivot candidates are ready without a dot product.  Each entry receives the
// same FMAs in the same order as the general kernel's left-looking update.
// Requires at most one owned row per thread (nrow - k0 - nbR <= threads).
// Columns go FP_COLS at a time through one exchange: the pivot W(c, c) is
// local, so every CTA can run the next columns' updates and candidate
// searches on the assumption that the earlier ones keep their diagonal
// pivots, and the exchange then returns all their column maxima.  The
// longest prefix that passes the test is kept; the global writes of a column
// (L, W, D) happen only once it is kept, so a stop leaves the later columns
// untouched for the general kernel.
// slot >= 0: one panel of a speculative batch -- kb goes to ctl->kb_log[slot]
// and an early stop sets ctl->halt, which makes every kernel queued after it
// return without work (the host replays from this panel).
__global__ void __launch_bounds__(FP_THREADS) k_wide_panel_fast(float *S, int nrow, int w, int k0, int nb,
                                                                float *Wb, int ldw, float *Dd, float *De,
                                                                WideCtl *ctl, int slot, int *status) {
  extern __shared__ __align__(16) unsigned char fp_raw[];
  __shared__ __align__(16) float wgrp[WP_NB * FP_COLS];  // W of a group's columns, rows of R
  if (*(volatile int *)&ctl->halt) return;  // queued behind a fast panel that stopped early
  const int nbR = min(nb, w - k0);  // panel columns = rows of R
  const int ldr = nbR + 1;
  float *sr = reinterpret_cast<float *>(fp_raw);  // [nbR][FP_THREADS]: the thread's row, panel columns
  float *Sr = sr + (size_t)nb * FP_THREADS;       // [nbR][ldr]: rows of R, W values once final
  const float alpha = (float)((1.0 + sqrt(17.0)) / 8.0);
  const int tid = threadIdx.x;
  const int gt = blockIdx.x * blockDim.x + tid;
  const int r_own = k0 + nbR + gt;  // the thread's row (if < nrow)
  const bool own = r_own < nrow;
  for (int e = tid; e < nbR * nbR; e += blockDim.x) {
    const int i = e % nbR, jj = e / nbR;
    Sr[i * ldr + jj] = i >= jj ? __ldcg(S + (k0 + i) + (size_t)(k0 + jj) * nrow) : 0.f;
  }
  if (own)
    for (int jj = 0; jj < nbR; ++jj) sr[jj * FP_THREADS + tid] = __ldcg(S + r_own + (size_t)(k0 + jj) * nrow);
  __syncthreads();
  // candidates of column 0
  unsigned hi = 0u, lo = 0u;
  auto consider = [&](float v, int r) {
    const float a = fabsf(v);
    const unsigned h = __float_as_uint(a), l = 0xFFFFFFu - (unsigned)r;
    if (a == a && (h > hi || (h == hi && l > lo))) {
      hi = h;
      lo = l;
    }
  };
  if (own && r_own < w) consider(sr[tid], r_own);
  if (tid >= 1 && tid < nbR && k0 + tid < w) consider(Sr[tid * ldr], k0 + tid);
  // rows of R: rank-1 term of local column jc on the lower triangle of the
  // trailing block (thread = row, column lane)
  auto rtri = [&](int jc) {
    const float r1 = 1.f / Sr[jc * ldr + jc];
    const int m = nbR - jc - 1, io = tid & 63, jl = tid >> 6;
    if (io < m) {
      const int i = jc + 1 + io;
      const float li = Sr[i * ldr + jc] * r1;
      for (int jo = jl; jo <= io; jo += FP_THREADS / 64) {
        const int jj = jc + 1 + jo;
        Sr[i * ldr + jj] = fmaf(-li, Sr[jj * ldr + jc], Sr[i * ldr + jj]);
      }
    }
  };
  // global writes of kept column jc (the thread's W value wv): L and W of the
  // thread's row, and (CTA 0) of the rows of R, the unit diagonal and D
  auto commit = [&](int jc, float wv) {
    const int c = k0 + jc;
    const float d = Sr[jc * ldr + jc];
    const float r1 = 1.f / d;
    if (own) {
      Wb[(size_t)jc * ldw + r_own] = wv;
      S[r_own + (size_t)c * nrow] = wv * r1;
    }
    if (blockIdx.x == 0) {
      for (int i = jc + tid; i < nbR; i += blockDim.x) {
        Wb[(size_t)jc * ldw + k0 + i] = Sr[i * ldr + jc];
        if (i > jc) S[(k0 + i) + (size_t)c * nrow] = Sr[i * ldr + jc] * r1;
      }
      if (tid == 0) {
        S[c + (size_t)c * nrow] = 1.f;
        Dd[c] = d;
        De[c] = 0.f;
      }
    }
  };
  // Columns go in groups of FP_COLS.  At a group's start the thread's row sr
  // carries the update of every earlier group; inside the group each column's
  // own entry gets the group's earlier columns as a short correction, and at
  // its end one rank-FP_COLS update (W of the group's columns as one float4 per
  // row of R) brings the rest of the row up to date.  Every entry receives
  // the same FMAs in the same order as a column-by-column update.
  unsigned epoch = 0;
  int j = 0;
  bool stop = false;
  while (j < nbR) {
    const int g = min(FP_COLS, nbR - j);
    float wq[FP_COLS] = {}, lq[FP_COLS] = {};  // the thread's W and L in the group's columns
    if (own) wq[0] = sr[j * FP_THREADS + tid];
    unsigned long long keys[FP_COLS] = {};
    keys[0] = cta_max_key(hi, lo);
    for (int q = 1; q < g; ++q) {
      lq[q - 1] = wq[q - 1] * (1.f / Sr[(j + q - 1) * ldr + j + q - 1]);
      hi = 0u;
      lo = 0u;
      if (own) {
        float v = sr[(j + q) * FP_THREADS + tid];
        for (int t = 0; t < q; ++t) v = fmaf(-lq[t], Sr[(j + q) * ldr + j + t], v);
        wq[q] = v;
        if (r_own < w) consider(v, r_own);
      }
      rtri(j + q - 1);
      __syncthreads();
      if (tid >= j + q + 1 && tid < nbR && k0 + tid < w) consider(Sr[tid * ldr + j + q], k0 + tid);
      keys[q] = cta_max_key(hi, lo);
    }
    unsigned long long best[FP_COLS];
    if (!grid_max_multi(ctl, epoch, keys, g, status, best)) return;
    int kept = 0;
    for (; kept < g; ++kept) {
      const float colmax = (float)__uint_as_float((unsigned)(best[kept] >> 24));
      const float absakk = fabsf(Sr[(j + kept) * ldr + j + kept]);
      if (!(absakk >= alpha * colmax) || absakk == 0.f) break;  // pivot search, zero or NaN pivot
    }
    for (int q = 0; q < kept; ++q) commit(j + q, wq[q]);
    if (kept < g) {
      j += kept;
      stop = true;  // the general kernel takes column k0 + j
      break;
    }
    const int jn = j + g;
    if (jn < nbR) {
      lq[g - 1] = wq[g - 1] * (1.f / Sr[(jn - 1) * ldr + jn - 1]);
      rtri(jn - 1);
      // W of the group's columns, rows jn .. nbR-1 of R (final: their last
      // term came from column jn - 2)
      for (int e = tid; e < (nbR - jn) * FP_COLS; e += blockDim.x) {
        const int i = jn + e / FP_COLS, q = e % FP_COLS;
        wgrp[i * FP_COLS + q] = q < g ? Sr[i * ldr + j + q] : 0.f;
      }
      __syncthreads();
      hi = 0u;
      lo = 0u;
      if (own) {
        for (int jj = jn; jj < nbR; ++jj) {
          const float4 wv = *reinterpret_cast<const float4 *>(wgrp + jj * FP_COLS);
          float v = sr[jj * FP_THREADS + tid];
          v = fmaf(-lq[0], wv.x, v);
          if (g > 1) v = fmaf(-lq[1], wv.y, v);
          if (g > 2) v = fmaf(-lq[2], wv.z, v);
          if (g > 3) v = fmaf(-lq[3], wv.w, v);
          sr[jj * FP_THREADS + tid] = v;
        }
        if (r_own < w) consider(sr[jn * FP_THREADS + tid], r_own);
      }
      if (tid >= jn + 1 && tid < nbR && k0 + tid < w) consider(Sr[tid * ldr + jn], k0 + tid);
    }
    j = jn;
  }
  if (blockIdx.x == 0 && tid == 0) {
    ctl->kb = j;
    ctl->stop = stop ? 1 : 0;
    if (slot >= 0) {
      ctl->kb_log[slot] = j;
      if (stop) ctl->halt = 1;
    }
  }
}

// Block-first fast panel (no pivot search).  The nbR x nbR diagonal block R
// is factored first, replicated in every CTA with diagonal pivots assumed,
// FB_RB columns at a time (one warp factors the diagonal block of the step
// with shuffles, the rows below it are solved against that block, then a
// rank-FB_RB update brings the rest of R up to date); then every owned row is solved
// against R in registers, and ONE grid exchange returns the maxima of all
// panel columns.  The longest prefix of columns whose diagonal passes the
// Bunch-Kaufman test is kept and written; the later columns stay untouched
// for the general kernel, as in k_wide_panel_fast.  Every entry receives the
// same FMAs in the same order as a column-by-column update, so both fast
// kernels give the same factor bit for bit.
// Exchange words: CTA b writes (maximum |W| bits of column j) << 32 | seq to
// word j * FB_MAXG + b of ctl->mslot; seq is unique per launch between two
// clearings of the control block, so the words need no clearing per launch.
constexpr int FB_THREADS = 256;  // one row below the panel per thread
constexpr int FB_MAXG = 128;     // CTAs per launch (WP_NB x FB_MAXG words fit in ctl->mslot)
constexpr int FB_LD = WP_NB;     // leading dimension of R, stored by columns
constexpr int FB_RB = 16;        // columns of R per blocked step
static_assert(WP_NB * FB_MAXG <= (int)(sizeof(WideCtl::mslot) / sizeof(unsigned long long)),
              "exchange words of the block-first panel");
static_assert(FB_THREADS % WP_NB == 0, "column parts of the exchange");

__host__ __device__ constexpr size_t fast_blk_smem() {
  return ((size_t)WP_NB * FB_THREADS + (size_t)WP_NB * FB_LD + FB_RB * FB_LD) * sizeof(float);
}

__global__ void __launch_bounds__(FB_THREADS) k_wide_panel_blk(float *S, int nrow, int w, int k0, int nb, float *Wb,
                                                               int ldw, float *Dd, float *De, WideCtl *ctl,
                                                               int slot, unsigned seq, int *status,
                                                               unsigned char *pack_a, unsigned char *pack_b,
                                                               int nkc_stride, int kcs, int pk_bf) {
  extern __shared__ __align__(16) unsigned char fb_raw[];
  __shared__ float rinv[WP_NB];
  __shared__ unsigned cpart[FB_THREADS / WP_NB][WP_NB];
  __shared__ int s_kept;
  if (*(volatile int *)&ctl->halt) return;  // queued behind a fast panel that stopped early
  const int nbR = min(nb, w - k0);           // panel columns = rows of R
  float *wsm = reinterpret_cast<float *>(fb_raw);  // [WP_NB][FB_THREADS]: W of the thread's row
  float *Rc = wsm + (size_t)WP_NB * FB_THREADS;    // [WP_NB][FB_LD]: R by columns, W values once final
  float *Lb = Rc + (size_t)WP_NB * FB_LD;          // [FB_RB][FB_LD]: L of the current column block
  const float alpha = (float)((1.0 + sqrt(17.0)) / 8.0);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int r_own = k0 + nbR + blockIdx.x * FB_THREADS + tid;  // the thread's row (if < nrow)
  const bool own = r_own < nrow;
  // R's lower triangle (zeros elsewhere), copied asynchronously
  for (int e = tid; e < WP_NB * FB_LD; e += FB_THREADS) {
    const int t = e / FB_LD, i = e % FB_LD;
    const bool in = t < nbR && i < nbR && i >= t;
    const float *src = in ? S + (k0 + i) + (size_t)(k0 + t) * nrow : S;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(Rc + e)),
                 "l"(src), "r"(in ? 4 : 0)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  if (tid < WP_NB) rinv[tid] = 0.f;
  // the thread's row, copied asynchronously so that the latency overlaps
  // the factorization of R (wsm[j][tid] is the thread's own column)
  if (own) {
    for (int j = 0; j < nbR; ++j)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(wsm + j * FB_THREADS + tid)),
                   "l"(S + r_own + (size_t)(k0 + j) * nrow)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  // R landed (the row copies may still be in flight)
  if (own) asm volatile("cp.async.wait_group 1;" ::: "memory");
  else asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  // --- R = L_R D_R L_R^T, FB_RB columns at a time -------------------------
  for (int b = 0; b < nbR; b += FB_RB) {
    const int nc = min(FB_RB, nbR - b);
    if (wid == 0) {
      // the FB_RB x FB_RB diagonal block: lane q holds row b + q
      const int q = lane;
      float v[FB_RB];
#pragma unroll
      for (int c = 0; c < FB_RB; ++c) v[c] = (q < nc && c <= q) ? Rc[(b + c) * FB_LD + b + q] : 0.f;
      // Every lane updates all its entries right of column t; those of its
      // strict upper part (c > q) and of lanes q >= nc are never read as
      // factor values nor stored, so no predicate is needed.
#pragma unroll
      for (int t = 0; t < FB_RB; ++t) {
        const float r1 = 1.f / __shfl_sync(0xffffffffu, v[t], t);
        const float l = v[t] * r1;
#pragma unroll
        for (int c = t + 1; c < FB_RB; ++c) {
          const float wct = __shfl_sync(0xffffffffu, v[t], c);  // W(b + c, b + t), final
          v[c] = fmaf(-l, wct, v[c]);
        }
        if (q == 0 && t < nc) rinv[b + t] = r1;
      }
#pragma unroll
      for (int c = 0; c < FB_RB; ++c)
        if (q < nc && c <= q) Rc[(b + c) * FB_LD + b + q] = v[c];
    }
    __syncthreads();
    const int mb = nbR - b - FB_RB;  // rows of R below the block (the block is full when > 0)
    if (mb <= 0) break;
    if (tid < mb) {
      const int i = b + FB_RB + tid;
      float v[FB_RB], lv[FB_RB];
#pragma unroll
      for (int c = 0; c < FB_RB; ++c) v[c] = Rc[(b + c) * FB_LD + i];
#pragma unroll
      for (int c = 0; c < FB_RB; ++c) {
#pragma unroll
        for (int t = 0; t < c; ++t) v[c] = fmaf(-lv[t], Rc[(b + t) * FB_LD + b + c], v[c]);
        lv[c] = v[c] * rinv[b + c];
      }
#pragma unroll
      for (int c = 0; c < FB_RB; ++c) {
        Rc[(b + c) * FB_LD + i] = v[c];
        Lb[c * FB_LD + i] = lv[c];
      }
    }
    __syncthreads();
    for (int e = tid; e < mb * mb; e += FB_THREADS) {
      const int io = e % mb, jo = e / mb;
      if (io < jo) continue;
      const int i = b + FB_RB + io, jj = b + FB_RB + jo;
      float x = Rc[jj * FB_LD + i];
#pragma unroll
      for (int t = 0; t < FB_RB; ++t) x = fmaf(-Lb[t * FB_LD + i], Rc[(b + t) * FB_LD + jj], x);
      Rc[jj * FB_LD + i] = x;
    }
    __syncthreads();
  }
  // --- the thread's row: forward substitution against R, 8 columns at a time
  if (own) {
    asm volatile("cp.async.wait_all;" ::: "memory");
    for (int jb = 0; jb < nbR; jb += 8) {
      const int nc = min(8, nbR - jb);
      float v[8], lv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = q < nc ? wsm[(jb + q) * FB_THREADS + tid] : 0.f;
      // (unrolled so that the shared-memory loads of several t overlap)
#pragma unroll 4
      for (int t = 0; t < jb; ++t) {
        const float l = wsm[t * FB_THREADS + tid] * rinv[t];
        const float4 x0 = *reinterpret_cast<const float4 *>(Rc + t * FB_LD + jb);
        const float4 x1 = *reinterpret_cast<const float4 *>(Rc + t * FB_LD + jb + 4);
        v[0] = fmaf(-l, x0.x, v[0]);
        v[1] = fmaf(-l, x0.y, v[1]);
        v[2] = fmaf(-l, x0.z, v[2]);
        v[3] = fmaf(-l, x0.w, v[3]);
        v[4] = fmaf(-l, x1.x, v[4]);
        v[5] = fmaf(-l, x1.y, v[5]);
        v[6] = fmaf(-l, x1.z, v[6]);
        v[7] = fmaf(-l, x1.w, v[7]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
#pragma unroll
        for (int t = 0; t < q; ++t) v[q] = fmaf(-lv[t], Rc[(jb + t) * FB_LD + jb + q], v[q]);
        lv[q] = v[q] * rinv[jb + q];
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nc) wsm[(jb + q) * FB_THREADS + tid] = v[q];
    }
  }
  __syncthreads();
  // --- column maxima: own rows inside the diagonal block and rows of R below
  // the diagonal, per CTA, then over the grid
  unsigned long long *slots = &ctl->mslot[0][0][0];
  const int nvalid = max(0, min(FB_THREADS, min(nrow, w) - (k0 + nbR + (int)blockIdx.x * FB_THREADS)));
  for (int j = wid; j < nbR; j += FB_THREADS / 32) {
    unsigned m = 0u;
#pragma unroll 4
    for (int t = lane; t < nvalid; t += 32) {
      const float a = fabsf(wsm[j * FB_THREADS + t]);
      if (a == a) m = max(m, __float_as_uint(a));
    }
    for (int i = j + 1 + lane; i < nbR; i += 32) {
      const float a = fabsf(Rc[j * FB_LD + i]);
      if (a == a) m = max(m, __float_as_uint(a));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0)
      *(volatile unsigned long long *)&slots[j * FB_MAXG + blockIdx.x] = ((unsigned long long)m << 32) | seq;
  }
  {
    const int G = (int)gridDim.x;
    const int q = tid % WP_NB, p = tid / WP_NB;
    long long it = 0;
    const long long lim_ = wait_limit(ctl);
    bool fail = false;
    // first every CTA's word of column 0, then every word (each re-checked)
    for (int phase = 0; phase < 2 && !fail; ++phase) {
      unsigned m = 0u;
      while (true) {
        bool all = true;
        m = 0u;
        if (phase == 0) {
          for (int bb = tid; bb < G; bb += FB_THREADS)
            if ((unsigned)*(volatile unsigned long long *)&slots[bb] != seq) all = false;
        } else if (q < nbR) {
          // all loads first (one L2 round trip), then the checks
          constexpr int NW = FB_MAXG / (FB_THREADS / WP_NB);
          unsigned long long v[NW];
#pragma unroll
          for (int k = 0; k < NW; ++k) {
            const int bb = p + k * (FB_THREADS / WP_NB);
            v[k] = bb < G ? *(volatile unsigned long long *)&slots[q * FB_MAXG + bb] : 0ull;
          }
#pragma unroll
          for (int k = 0; k < NW; ++k) {
            if (p + k * (FB_THREADS / WP_NB) >= G) continue;
            if ((unsigned)v[k] != seq) all = false;
            else m = max(m, (unsigned)(v[k] >> 32));
          }
        }
        if (__syncthreads_and(all)) break;
        const int ab = tid == 0 ? *(volatile int *)&ctl->abort : 0;
        if (__syncthreads_or(ab)) {
          fail = true;
          break;
        }
        if (++it > lim_) {
          if (tid == 0) {
            atomicOr(status, ST_TIMEOUT);
            atomicExch(&ctl->abort, 1);
          }
          fail = true;
          break;
        }
      }
      if (phase == 1) cpart[p][q] = m;
    }
    if (fail) return;
    __syncthreads();
  }
  if (tid == 0) {
    int k = 0;
    for (; k < nbR; ++k) {
      unsigned mb = 0u;
#pragma unroll
      for (int p = 0; p < FB_THREADS / WP_NB; ++p) mb = max(mb, cpart[p][k]);
      const float colmax = __uint_as_float(mb);
      const float absakk = fabsf(Rc[k * FB_LD + k]);
      if (!(absakk >= alpha * colmax) || absakk == 0.f) break;  // pivot search, zero or NaN pivot
    }
    s_kept = k;
  }
  __syncthreads();
  // --- global writes of the kept columns
  const int kept = s_kept;
  // W goes to Wb only where a later kernel reads it there: without packed
  // operands, or for a short panel (its operands are packed again from Wb)
  const bool wb_out = !pack_a || kept < nbR;
  if (own)
    for (int j = 0; j < kept; ++j) {
      const float wv = wsm[j * FB_THREADS + tid];
      if (wb_out) Wb[(size_t)j * ldw + r_own] = wv;
      S[r_own + (size_t)(k0 + j) * nrow] = wv * rinv[j];
    }
  // operands of the trailing updates (pack_a non-null): the thread's row of
  // L (A) and, inside the diagonal block, of W (B) as split blocks (TF32, or
  // BF16 when pk_bf) in the layout of k_pack_split, chunks kcs .. of row
  // block r_own / 128, columns from kept on zero.  Rows of the panel itself
  // are never read by a later update (they lie above every updated column)
  // and are not written.
  if (pack_a && own) {
    const int rb = r_own / t5::TM, rr = r_own % t5::TM;
    auto pack_row = [&](auto bf_tag) {
      constexpr bool BF = decltype(bf_tag)::value;
      constexpr int KC = pk_chunk(BF), UE = KC / 8;
      for (int c = 0; c * KC < nbR; ++c) {
        const size_t blk = ((size_t)rb * nkc_stride + kcs + c) * (2 * t5::OPND_BYTES);
        unsigned char *ah = pack_a + blk, *bh = r_own < w ? pack_b + blk : nullptr;
#pragma unroll 2
        for (int cc = 0; cc < 8; ++cc) {
          float lx[UE], wx[UE];
#pragma unroll
          for (int q = 0; q < UE; ++q) {
            const int j = c * KC + cc * UE + q;
            const float wv = j < kept ? wsm[j * FB_THREADS + tid] : 0.f;
            wx[q] = wv;
            lx[q] = j < kept ? wv * rinv[j] : 0.f;
          }
          pk_store_unit<BF>(ah, ah + t5::OPND_BYTES, rr, cc, lx);
          if (bh) pk_store_unit<BF>(bh, bh + t5::OPND_BYTES, rr, cc, wx);
        }
      }
    };
    if (pk_bf) pack_row(std::true_type{});
    else pack_row(std::false_type{});
  }
  if (blockIdx.x == 0) {
    for (int e = tid; e < kept * nbR; e += FB_THREADS) {
      const int j = e / nbR, i = e % nbR;
      if (i < j) continue;
      const float v = Rc[j * FB_LD + i];
      const int c = k0 + j;
      if (wb_out) Wb[(size_t)j * ldw + k0 + i] = v;
      if (i > j) {
        S[(k0 + i) + (size_t)c * nrow] = v * rinv[j];
      } else {
        S[c + (size_t)c * nrow] = 1.f;
        Dd[c] = v;
        De[c] = 0.f;
      }
    }
    if (tid == 0) {
      ctl->kb = kept;
      ctl->stop = kept < nbR ? 1 : 0;
      if (slot >= 0) {
        ctl->kb_log[slot] = kept;
        if (kept < nbR) ctl->halt = 1;
      }
    }
  }
}

// One panel: columns c = k0 .. (at most k0+nb, one more for a final 2x2).
// Thread gt owns rows gt, gt + TT, ...; the panel entries L(gt, k0 + t) of
// its first row are cached in shared memory (lc[t][threadIdx.x]) as they are
// produced, and its W entries stay in registers, so the column updates read
// no global memory for that row.  After each column's exchange one round of
// loads brings the pivot W(c, j), the next column's own entry S(gt, c+1) and
// the row W(c+1, 0..j) of the next update; a pivot search or an interchange
// (rare once the pivot order has settled) reloads what it changed.
template <class T>
__global__ void __launch_bounds__(WP_THREADS) k_wide_panel(T *S, int nrow, int w, int k0, int nb, T *Wb, int ldw,
                                                           T *Dd, T *De, int *perm, WideCtl *ctl, int *status) {
  extern __shared__ __align__(16) unsigned char wp_raw[];
  T *lc = reinterpret_cast<T *>(wp_raw);  // [WP_NB + 2][WP_THREADS]
  __shared__ T wbuf[2][WP_NB + 2];        // W(c, 0..j-1) of the current column, and of the next
  __shared__ T wrB[WP_NB + 2];            // W(imax, 0..j-1) of a pivot-row update
  const T alpha = (T)((1.0 + sqrt(17.0)) / 8.0);
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int TT = gridDim.x * blockDim.x;
  const int tid = threadIdx.x;
  auto first_row = [&](int lo) { return lo + (int)(((long long)gt - lo % TT + TT) % TT); };
  unsigned epoch = 0;
  int cur = 0;  // wbuf[cur] holds W(c, 0..j-1)
  T s_own = (gt >= k0 && gt < nrow && k0 < w) ? __ldcg(S + gt + (size_t)k0 * nrow) : T(0);
  int j = 0;
  while (j < nb && k0 + j < w) {
    const int c = k0 + j;
    const T *wrow = wbuf[cur];
    // ---- A: updated column c into W(:, j), rows [c, nrow)
    T cv = T(-1), w_own = T(0);
    int ci = -1;
    for (int r = first_row(c); r < nrow; r += TT) {
      T acc;
      if (r == gt) {
        acc = s_own;
        for (int t = 0; t < j; ++t) acc -= lc[t * WP_THREADS + tid] * wrow[t];
        w_own = acc;
      } else {
        acc = __ldcg(S + r + (size_t)c * nrow);
        for (int t = 0; t < j; ++t) acc -= __ldcg(S + r + (size_t)(k0 + t) * nrow) * wrow[t];
      }
      Wb[(size_t)j * ldw + r] = acc;
      if (r > c && r < w) {
        const T a = tabs_w(acc);
        if (a == a && (ci < 0 || a > cv)) {
          cv = a;
          ci = r;
        }
      }
    }
    T colmax;
    int imax;
    if (!grid_argmax(cv, ci, ctl, 0, epoch, status, colmax, imax)) return;
    if (imax < 0) colmax = T(0);
    // one round of loads: pivot, and the next column's inputs on the fast path
    const T wcc = __ldcg(Wb + (size_t)j * ldw + c);
    T *wnext = wbuf[cur ^ 1];
    if (tid <= j && c + 1 < nrow) wnext[tid] = __ldcg(Wb + (size_t)tid * ldw + c + 1);
    const T s_next = (gt >= c + 1 && gt < nrow && c + 1 < w) ? __ldcg(S + gt + (size_t)(c + 1) * nrow) : T(0);
    const T absakk = tabs_w(wcc);
    int kp = c, kstep = 1;
    bool zero = false, slow = false;
    T w_own1 = T(0);
    if ((absakk >= colmax ? absakk : colmax) == T(0) || absakk != absakk) {
      zero = true;
    } else if (absakk < alpha * colmax) {
      slow = true;
      // ---- B: updated column imax into W(:, j+1) and its off-diagonal max
      for (int t = tid; t < j; t += blockDim.x) wrB[t] = __ldcg(Wb + (size_t)t * ldw + imax);
      __syncthreads();
      T rv = T(-1);
      int ri = -1;
      for (int r = first_row(c); r < nrow; r += TT) {
        T acc = r < imax ? __ldcg(S + imax + (size_t)r * nrow) : __ldcg(S + r + (size_t)imax * nrow);
        if (r == gt) {
          for (int t = 0; t < j; ++t) acc -= lc[t * WP_THREADS + tid] * wrB[t];
          w_own1 = acc;
        } else {
          for (int t = 0; t < j; ++t) acc -= __ldcg(S + r + (size_t)(k0 + t) * nrow) * wrB[t];
        }
        Wb[(size_t)(j + 1) * ldw + r] = acc;
        if (r < w && r != imax) {
          const T a = tabs_w(acc);
          if (a == a && (ri < 0 || a > rv)) {
            rv = a;
            ri = r;
          }
        }
      }
      T rowmax;
      int rdummy;
      if (!grid_argmax(rv, ri, ctl, 1, epoch, status, rowmax, rdummy)) return;
      const T diag_imax = tabs_w(__ldcg(Wb + (size_t)(j + 1) * ldw + imax));
      if (absakk >= alpha * colmax * (colmax / rowmax)) {
        kp = c;
      } else if (diag_imax >= alpha * rowmax) {
        kp = imax;
      } else {
        kp = imax;
        kstep = 2;
      }
    }
    const int kk = c + kstep - 1;
    // ---- C: interchange kk <-> kp
    if (kp != kk) {
      const bool copycol = (kstep == 1);  // working column becomes the updated column kp
      for (int r = first_row(c); r < nrow; r += TT) {
        if (copycol && r != kk && r != kp) {
          const T v1 = __ldcg(Wb + (size_t)(j + 1) * ldw + r);
          Wb[(size_t)j * ldw + r] = v1;
        }
        if (r > kp) {
          T t = __ldcg(S + r + (size_t)kk * nrow);
          S[r + (size_t)kk * nrow] = __ldcg(S + r + (size_t)kp * nrow);
          S[r + (size_t)kp * nrow] = t;
        } else if (r > kk && r < kp) {
          T t = __ldcg(S + r + (size_t)kk * nrow);
          S[r + (size_t)kk * nrow] = __ldcg(S + kp + (size_t)r * nrow);
          S[kp + (size_t)r * nrow] = t;
        }
      }
      for (int col = gt; col < kk; col += TT) {  // rows kk, kp of all finished columns
        T t = __ldcg(S + kk + (size_t)col * nrow);
        S[kk + (size_t)col * nrow] = __ldcg(S + kp + (size_t)col * nrow);
        S[kp + (size_t)col * nrow] = t;
      }
      if (gt == 0) {
        T t = __ldcg(S + kk + (size_t)kk * nrow);
        S[kk + (size_t)kk * nrow] = __ldcg(S + kp + (size_t)kp * nrow);
        S[kp + (size_t)kp * nrow] = t;
        int pt = perm[kk];
        perm[kk] = perm[kp];
        perm[kp] = pt;
        if (copycol) {
          T a1 = __ldcg(Wb + (size_t)(j + 1) * ldw + kp), a2 = __ldcg(Wb + (size_t)(j + 1) * ldw + kk);
          Wb[(size_t)j * ldw + kk] = a1;
          Wb[(size_t)j * ldw + kp] = a2;
          for (int t2 = 0; t2 < j; ++t2) {
            T x = __ldcg(Wb + (size_t)t2 * ldw + kk);
            Wb[(size_t)t2 * ldw + kk] = __ldcg(Wb + (size_t)t2 * ldw + kp);
            Wb[(size_t)t2 * ldw + kp] = x;
          }
        } else {
          for (int t2 = 0; t2 <= j + 1; ++t2) {
            T x = __ldcg(Wb + (size_t)t2 * ldw + kk);
            Wb[(size_t)t2 * ldw + kk] = __ldcg(Wb + (size_t)t2 * ldw + kp);
            Wb[(size_t)t2 * ldw + kp] = x;
          }
        }
        ctl->pivoted = 1;
      }
      unsigned long long dummy;
      if (!grid_exchange(ctl, epoch, 0ull, status, dummy)) return;
      if (gt == kk || gt == kp)
        for (int t = 0; t < j; ++t) lc[t * WP_THREADS + tid] = __ldcg(S + gt + (size_t)(k0 + t) * nrow);
    }
    if (slow && gt < nrow) {
      // W entries of the thread's own row after the pivot search / interchange
      w_own = __ldcg(Wb + (size_t)j * ldw + gt);
      w_own1 = __ldcg(Wb + (size_t)(j + 1) * ldw + gt);
    }
    // ---- D: L column(s) from W, D entries
    if (kstep == 1) {
      const T d = slow ? __ldcg(Wb + (size_t)j * ldw + c) : wcc;
      const T r1 = zero ? T(1) : T(1) / d;
      for (int r = first_row(c + 1); r < nrow; r += TT) {
        const T wv = r == gt ? w_own : __ldcg(Wb + (size_t)j * ldw + r);
        // zero pivot column: kept unscaled (LAPACK dlasyf copies W(k:n,k))
        const T l = zero ? wv : wv * r1;
        S[r + (size_t)c * nrow] = l;
        if (r == gt) lc[j * WP_THREADS + tid] = l;
      }
      if (gt == 0) {
        if (zero && absakk == absakk) atomicOr(status, ST_ZERO_PIVOT);
        S[c + (size_t)c * nrow] = T(1);
        Dd[c] = d;
        De[c] = T(0);
      }
    } else {
      const T D11 = __ldcg(Wb + (size_t)j * ldw + c), D21 = __ldcg(Wb + (size_t)j * ldw + c + 1);
      const T D22 = __ldcg(Wb + (size_t)(j + 1) * ldw + c + 1);
      T d21 = D21;
      const T d11 = D22 / d21, d22 = D11 / d21;
      const T tt = T(1) / (d11 * d22 - T(1));
      d21 = tt / d21;
      for (int r = first_row(c + 2); r < nrow; r += TT) {
        const T wk = r == gt ? w_own : __ldcg(Wb + (size_t)j * ldw + r);
        const T wk1 = r == gt ? w_own1 : __ldcg(Wb + (size_t)(j + 1) * ldw + r);
        const T l0 = d21 * (d11 * wk - wk1), l1 = d21 * (d22 * wk1 - wk);
        S[r + (size_t)c * nrow] = l0;
        S[r + (size_t)(c + 1) * nrow] = l1;
        if (r == gt) {
          lc[j * WP_THREADS + tid] = l0;
          lc[(j + 1) * WP_THREADS + tid] = l1;
        }
      }
      if (gt == 0) {
        S[c + (size_t)c * nrow] = T(1);
        S[c + 1 + (size_t)(c + 1) * nrow] = T(1);
        S[c + 1 + (size_t)c * nrow] = T(0);
        Dd[c] = D11;
        Dd[c + 1] = D22;
        De[c] = D21;
        De[c + 1] = T(0);
      }
    }
    j += kstep;
    const int cn = k0 + j;
    if (!slow) {
      // fast path: no interchange, next column is c + 1
      s_own = s_next;
      cur ^= 1;
      __syncthreads();
    } else if (j < nb && cn < w) {
      // reload the next column's inputs after the pivot search / interchange
      __syncthreads();
      if (tid < j) wbuf[cur][tid] = __ldcg(Wb + (size_t)tid * ldw + cn);
      s_own = (gt >= cn && gt < nrow) ? __ldcg(S + gt + (size_t)cn * nrow) : T(0);
      __syncthreads();
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->kb = j;
}

// A22 -= L21 W21^T for rows [k1, nrow) and columns [k1, w), lower part of the
// diagonal block only.  L21 = S(:, k0..k0+kb), W21 = Wb(:, 0..kb).
template <class T, int BM, int BN, int RM, int RN>
__global__ void __launch_bounds__((BM / RM) * (BN / RN)) k_wide_trailing(T *S, int nrow, int w, int k0, int kb,
                                                                        const T *Wb, int ldw, int tiles_n) {
  constexpr int KC = 16;
  constexpr int TX = BN / RN, TY = BM / RM, NT = TX * TY;
  __shared__ T As[KC][BM + 4];
  __shared__ T Bs[KC][BN + 4];
  const int k1 = k0 + kb;
  const int tn = blockIdx.x % tiles_n, tm = blockIdx.x / tiles_n;
  const int col0 = k1 + tn * BN;
  const int row0 = k1 + tm * BM;
  if (row0 + BM - 1 < col0) return;  // tile strictly above the diagonal
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  T acc[RM][RN];
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int b = 0; b < RN; ++b) acc[a][b] = T(0);
  for (int t0 = 0; t0 < kb; t0 += KC) {
    __syncthreads();
    for (int e = tid; e < KC * BM; e += NT) {
      int cc = e / BM, i = e % BM;
      int t = t0 + cc, r = row0 + i;
      As[cc][i] = (t < kb && r < nrow) ? S[r + (size_t)(k0 + t) * nrow] : T(0);
    }
    for (int e = tid; e < KC * BN; e += NT) {
      int cc = e / BN, q = e % BN;
      int t = t0 + cc, col = col0 + q;
      Bs[cc][q] = (t < kb && col < w) ? Wb[(size_t)t * ldw + col] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int cc = 0; cc < KC; ++cc) {
      T av[RM], bv[RN];
#pragma unroll
      for (int a = 0; a < RM; ++a) av[a] = As[cc][ty + a * TY];
#pragma unroll
      for (int b = 0; b < RN; ++b) bv[b] = Bs[cc][tx + b * TX];
#pragma unroll
      for (int a = 0; a < RM; ++a)
#pragma unroll
        for (int b = 0; b < RN; ++b) acc[a][b] += av[a] * bv[b];
    }
  }
#pragma unroll
  for (int a = 0; a < RM; ++a) {
    const int r = row0 + ty + a * TY;
    if (r >= nrow) continue;
#pragma unroll
    for (int b = 0; b < RN; ++b) {
      const int col = col0 + tx + b * TX;
      if (col >= w || r < col) continue;
      S[r + (size_t)col * nrow] -= acc[a][b];
    }
  }
}

// FP32 trailing update on tensor cores: the same A22 -= L21 W21^T as
// k_wide_trailing, with split-TF32 mma.sync products (FP32-level accuracy).
// CTA tile 128 x 128, eight warps of 64 x 32; K in chunks of 32 staged
// column-major in shared memory (conflict-free fragment reads with a leading
// dimension of 136); the result is staged through shared memory so that the
// read-modify-write of the factor is coalesced along its columns.
constexpr int TC_BM = 128, TC_BN = 128, TC_KC = 32, TC_LD = 136, TC_LDC = 132;
constexpr size_t TC_SMEM = (size_t)TC_BN * TC_LDC * sizeof(float);  // >= 2 * TC_KC * TC_LD floats

__global__ void __launch_bounds__(256, 2) k_wide_trailing_tc(float *S, int nrow, int w, int k0, int kb,
                                                              const float *Wb, int ldw, int tiles_n) {
  extern __shared__ __align__(16) float tc_smem[];
  float *As = tc_smem;                 // [TC_KC][TC_LD]: L21 rows of the tile
  float *Bs = tc_smem + TC_KC * TC_LD;  // [TC_KC][TC_LD]: W21 rows (= factor columns) of the tile
  const int k1 = k0 + kb;
  const int tn = blockIdx.x % tiles_n, tm = blockIdx.x / tiles_n;
  const int col0 = k1 + tn * TC_BN;
  const int row0 = k1 + tm * TC_BM;
  if (row0 + TC_BM - 1 < col0) return;  // tile strictly above the diagonal
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3, g = lane >> 2, t = lane & 3;
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int jn = 0; jn < 4; ++jn)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][jn][q] = 0.f;
  for (int kc0 = 0; kc0 < kb; kc0 += TC_KC) {
    __syncthreads();
    for (int e = tid; e < TC_KC * TC_BM; e += 256) {
      const int kk = e / TC_BM, i = e % TC_BM;
      const int kt = kc0 + kk, r = row0 + i, col = col0 + i;
      As[kk * TC_LD + i] = (kt < kb && r < nrow) ? S[r + (size_t)(k0 + kt) * nrow] : 0.f;
      Bs[kk * TC_LD + i] = (kt < kb && col < w) ? Wb[(size_t)kt * ldw + col] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < TC_KC; ks += 8) {
      uint32_t ah[4][4], al[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int rb = wm * 64 + i * 16 + g;
        split_tf32(As[(ks + t) * TC_LD + rb], ah[i][0], al[i][0]);
        split_tf32(As[(ks + t) * TC_LD + rb + 8], ah[i][1], al[i][1]);
        split_tf32(As[(ks + t + 4) * TC_LD + rb], ah[i][2], al[i][2]);
        split_tf32(As[(ks + t + 4) * TC_LD + rb + 8], ah[i][3], al[i][3]);
      }
#pragma unroll
      for (int jn = 0; jn < 4; ++jn) {
        const int cb = wn * 32 + jn * 8 + g;
        uint32_t bh[2], bl[2];
        split_tf32(Bs[(ks + t) * TC_LD + cb], bh[0], bl[0]);
        split_tf32(Bs[(ks + t + 4) * TC_LD + cb], bh[1], bl[1]);
#pragma unroll
        for (int i = 0; i < 4; ++i) mma_tf32x3(acc[i][jn], ah[i], al[i], bh, bl);
      }
    }
  }
  __syncthreads();
  float *Cs = tc_smem;  // [TC_BN][TC_LDC], column-major tile of the product
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int jn = 0; jn < 4; ++jn) {
      const int r = wm * 64 + i * 16 + g, c = wn * 32 + jn * 8 + 2 * t;
      Cs[c * TC_LDC + r] = acc[i][jn][0];
      Cs[(c + 1) * TC_LDC + r] = acc[i][jn][1];
      Cs[c * TC_LDC + r + 8] = acc[i][jn][2];
      Cs[(c + 1) * TC_LDC + r + 8] = acc[i][jn][3];
    }
  __syncthreads();
  // read-modify-write in batches of 8 columns: the loads of a batch are issued
  // before its stores (they cannot be reordered across stores to the factor)
  const int r = tid & (TC_BM - 1), gr = row0 + r;
  for (int cb = (tid >> 7) * 8; cb < TC_BN; cb += 16) {
    float cur[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int gc = col0 + cb + q;
      cur[q] = (gr < nrow && gc < w && gr >= gc) ? S[gr + (size_t)gc * nrow] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int gc = col0 + cb + q;
      if (gr < nrow && gc < w && gr >= gc) S[gr + (size_t)gc * nrow] = cur[q] - Cs[(cb + q) * TC_LDC + r];
    }
  }
}

// FP32 trailing update on the fifth-generation tensor cores: one 128 x 128
// tile of A22 -= L21 W21^T per CTA of four warps, split-TF32 products
// accumulated in TMEM (tile_tf32x3, one operand stage so that three CTAs share
// an SM), and a read-modify-write epilogue in which thread r owns row r of the
// tile (coalesced along the factor's columns).
// Columns [cbeg, w) (rows from cbeg, lower part) receive the update of the
// kb factor columns starting at kL, whose W = L D columns are Wb[0..kb).
__global__ void __launch_bounds__(t5::THREADS) k_wide_trailing_t5(float *S, int nrow, int kL, int kb, int cbeg,
                                                                  int w, const float *Wb, int ldw, int tiles_n,
                                                                  const int *halt, int *status) {
  extern __shared__ __align__(1024) unsigned char t5_smem[];
  if (*(volatile const int *)halt) return;  // queued behind a fast panel that stopped early
  const int tn = blockIdx.x % tiles_n, tm = blockIdx.x / tiles_n;
  const int col0 = cbeg + tn * t5::TN;
  const int row0 = cbeg + tm * t5::TM;
  if (row0 + t5::TM - 1 < col0) return;  // tile strictly above the diagonal
  const float *L21 = S + (size_t)kL * nrow;
  auto fa = [&](int r, int k0c, float(&x)[t5::TK]) {
    const int gr = row0 + r;
#pragma unroll
    for (int k = 0; k < t5::TK; ++k)
      x[k] = (gr < nrow && k0c + k < kb) ? L21[gr + (size_t)(k0c + k) * nrow] : 0.f;
  };
  auto fb = [&](int n, int k0c, float(&x)[t5::TK]) {
    const int gc = col0 + n;
#pragma unroll
    for (int k = 0; k < t5::TK; ++k) x[k] = (gc < w && k0c + k < kb) ? Wb[(size_t)(k0c + k) * ldw + gc] : 0.f;
  };
  auto ep = [&](int r, int c0, const uint32_t(&v)[32]) {
    const int gr = row0 + r;
    if (gr >= nrow) return;
    float cur[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int gc = col0 + c0 + q;
      cur[q] = (gc < w && gr >= gc) ? S[gr + (size_t)gc * nrow] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int gc = col0 + c0 + q;
      if (gc < w && gr >= gc) S[gr + (size_t)gc * nrow] = cur[q] - __uint_as_float(v[q]);
    }
  };
  t5::tile_tf32x3<1>(kb, fa, fb, ep, t5_smem, status);
}

// ---------------------------------------------------------------------------
// Persistent trailing update on the tcgen05 tensor cores.
//
// Operands are packed once per panel: k_pack_split writes the panel's L rows
// (A) and W rows (B) as split blocks of 128 rows x one chunk of K (64 BF16 or
// 32 TF32 entries; hi then lo, 16 KB each, in the swizzled K-major layout of
// t5::store_row_split), block (rb, kc) at rb * nkc_stride + kc, row blocks at
// absolute 128-row positions of the supernode, every panel starting on a new
// chunk (zeros pad a partial chunk).  k_tc_persistent then runs one CTA
// per SM over the lower-triangular set of 128 x 128 tiles: warp 0 streams
// both operand blocks of each K chunk into a three-stage shared-memory ring
// with bulk copies, warp 1 issues the split MMAs (lo.hi, hi.lo, hi.hi per
// 32-byte K step, as t5::tile_tf32x3) into one of two TMEM accumulators,
// and warps 2-9 (two per TMEM lane quarter, 64 columns each) subtract the
// finished accumulator from S while the next tile accumulates in the other
// one; they load their S values before the accumulator is ready.
constexpr int PK_BLOCK = 2 * t5::OPND_BYTES;  // hi + lo of one 128-row block of a chunk
constexpr int TP_STAGES = 3;
constexpr int TP_THREADS = 320;  // producer warp, MMA warp, 8 epilogue warps

__host__ __device__ constexpr size_t tp_smem_bytes() { return (size_t)TP_STAGES * t5::STAGE_BYTES + 1024; }

// Blocks of rows [rb_first * 128, row_hi) x columns [0, kb) of src (element
// (r, k) at src[r + k * ld]) into chunks kc0 .. of the pack buffer (a chunk
// holds pk_chunk(BF) columns).
template <bool BF>
__global__ void __launch_bounds__(256) k_pack_split(const float *src, int ld, int row_hi, int kb, unsigned char *dst,
                                                    int nkc_stride, int kc0, int rb_first, const int *halt) {
  constexpr int KC = pk_chunk(BF), UE = KC / 8;  // K per chunk, entries per 16-byte unit
  __shared__ float tk[KC][t5::TM + 1];
  if (halt && *(volatile const int *)halt) return;  // queued behind a fast panel that stopped early
  const int rb = rb_first + blockIdx.x, kcl = blockIdx.y;
  const int r0 = rb * t5::TM, k0 = kcl * KC;
  for (int e = threadIdx.x; e < KC * t5::TM; e += blockDim.x) {
    const int k = e / t5::TM, r = e % t5::TM, gr = r0 + r;
    tk[k][r] = (gr < row_hi && k0 + k < kb) ? __ldcg(src + gr + (size_t)(k0 + k) * ld) : 0.f;
  }
  __syncthreads();
  unsigned char *hi = dst + ((size_t)rb * nkc_stride + kc0 + kcl) * PK_BLOCK, *lo = hi + t5::OPND_BYTES;
  const int r = threadIdx.x >> 1;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int c = (threadIdx.x & 1) * 4 + cc;
    float x[UE];
#pragma unroll
    for (int q = 0; q < UE; ++q) x[q] = tk[UE * c + q][r];
    pk_store_unit<BF>(hi, lo, r, c, x);
  }
}

// Split-TF32 blocks of (L D)(i, k) = d_k L(i, k) + e_k L(i, k+1) + e_{k-1}
// L(i, k-1) for rows [0, row_hi) and columns [0, kb) of src (element (i, t)
// at src[i + t * ld]; d, e the descendant's diagonal and 2 x 2 sub-diagonal),
// in the layout of k_pack_split, chunk kc of row block rb at rb * nkc + kc.
template <bool BF>
__global__ void __launch_bounds__(256) k_pack_ld(const float *src, int ld, int row_hi, int kb, const float *Dd,
                                                 const float *Ed, unsigned char *dst, int nkc) {
  constexpr int KC = pk_chunk(BF), UE = KC / 8;
  __shared__ float tk[KC + 2][t5::TM + 1];
  const int rb = blockIdx.x, kc = blockIdx.y;
  const int r0 = rb * t5::TM, k0 = kc * KC;
  for (int e = threadIdx.x; e < (KC + 2) * t5::TM; e += blockDim.x) {
    const int q = e / t5::TM, r = e % t5::TM, t = k0 - 1 + q, gr = r0 + r;
    tk[q][r] = (gr < row_hi && t >= 0 && t < kb) ? __ldcg(src + gr + (size_t)t * ld) : 0.f;
  }
  __syncthreads();
  unsigned char *hi = dst + ((size_t)rb * nkc + kc) * PK_BLOCK, *lo = hi + t5::OPND_BYTES;
  const int r = threadIdx.x >> 1;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int c = (threadIdx.x & 1) * 4 + cc;
    float x[UE];
#pragma unroll
    for (int q = 0; q < UE; ++q) {
      const int k = UE * c + q, t = k0 + k;
      const float dk = t < kb ? Dd[t] : 0.f, ek = t < kb ? Ed[t] : 0.f;
      const float em = (t >= 1 && t - 1 < kb) ? Ed[t - 1] : 0.f;
      x[q] = dk * tk[k + 1][r] + ek * tk[k + 2][r] + em * tk[k][r];
    }
    pk_store_unit<BF>(hi, lo, r, c, x);
  }
}

// Target positions of a descendant pair: row i (< m) of the pair's rows goes
// to row prow[i] of the target supernode (cs0, ws columns, nrs rows listed in
// rows_s), column j (< nc) to column pcol[j]; -1 and ST_BOUNDS when absent.
__global__ void k_pair_map(const int *rows, int m, int nc, const int *rows_s, int nrs, int cs0, int ws, int *prow,
                           int *pcol, int *status) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const int r = rows[i];
    int pos;
    if (r < cs0 + ws) {
      pos = r - cs0;
    } else {
      int lo = ws, hi = nrs;  // first listed row >= r
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (rows_s[mid] < r) lo = mid + 1;
        else hi = mid;
      }
      pos = (lo < nrs && rows_s[lo] == r) ? lo : -1;
    }
    if (pos < 0) atomicOr(status, ST_BOUNDS);
    prow[i] = pos;
    if (i < nc) {
      const int c = r - cs0;
      const bool ok = c >= 0 && c < ws;
      if (!ok) atomicOr(status, ST_BOUNDS);
      pcol[i] = ok ? c : -1;
    }
  }
}

// Tile t of the lower-triangular tile set: column block c holds row blocks
// c .. nrb-1 (both relative to the first block).
__device__ __forceinline__ void tp_tile(int t, int nrb, int ncb, int &rbl, int &cbl) {
  int lo = 0, hi = ncb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const long long o = (long long)mid * nrb - (long long)mid * (mid - 1) / 2;
    if (o <= t) lo = mid;
    else hi = mid - 1;
  }
  cbl = lo;
  rbl = lo + (int)(t - ((long long)lo * nrb - (long long)lo * (lo - 1) / 2));
}

// Tiles in groups of TP_GB x TP_GB blocks (lower-triangular set of groups,
// by columns; tiles inside a group by columns): the CTAs of one wave work on
// about TP_GB row blocks and TP_GB column blocks, so that each operand block
// comes from DRAM once per group and from L2 for the other tiles of the
// group.  Flat index t covers every position of every group; positions
// outside the tile set return false.
constexpr int TP_GB = 12;
__host__ __device__ constexpr long long tp_flat_count(int nrb, int ncb) {
  return (((long long)(ncb + TP_GB - 1) / TP_GB) * ((nrb + TP_GB - 1) / TP_GB) -
          ((long long)(ncb + TP_GB - 1) / TP_GB) * ((ncb + TP_GB - 1) / TP_GB - 1) / 2) *
         TP_GB * TP_GB;
}
__device__ __forceinline__ bool tp_tile_grouped(int t, int nrb, int ncb, int &rbl, int &cbl) {
  const int gidx = t / (TP_GB * TP_GB), l = t % (TP_GB * TP_GB);
  int gi, gj;
  tp_tile(gidx, (nrb + TP_GB - 1) / TP_GB, (ncb + TP_GB - 1) / TP_GB, gi, gj);
  rbl = gi * TP_GB + l % TP_GB;
  cbl = gj * TP_GB + l / TP_GB;
  return rbl < nrb && cbl < ncb && rbl >= cbl;
}

// Bounded mbarrier wait that also gives up once another role has given up.
__device__ __forceinline__ bool tp_wait(uint32_t mbar, uint32_t parity, volatile int *abort, int *status) {
  for (long long it = 0; it < t5::WAIT_LIMIT; ++it) {
    if (t5::mbar_test(mbar, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  atomicOr(status, ST_TIMEOUT);
  return false;
}

// Sum over chunks kc0 .. kc1-1 of A(i, :) B(j, :)^T for the tiles of blocks
// blk0 + (rbl, cbl) (ntile: tiles, or tp_flat_count positions when MAPPED),
// subtracted from S:
//   MAPPED = false (trailing update, S column-major with leading dimension
//     nrow): at S[i, j] for j in [cb, ce), i >= j, i < nrow;
//   MAPPED = true (descendant pair, i, j relative to its first row): at
//     S[prow[i] + pcol[j] * nrow] for i < mrows, j < ncols, j <= i.
template <bool MAPPED, bool BF>
__global__ void __launch_bounds__(TP_THREADS, 1) k_tc_persistent(float *S, int nrow, int cb, int ce,
                                                                 const unsigned char *pack_a,
                                                                 const unsigned char *pack_b, int nkc_stride, int kc0,
                                                                 int kc1, int blk0, int nrb, int ncb, int ntile,
                                                                 const int *halt, int *status, const int *prow,
                                                                 const int *pcol, int mrows, int ncols) {
  extern __shared__ __align__(1024) unsigned char tp_raw[];
  __shared__ __align__(8) uint64_t bar[2 * TP_STAGES + 4];
  // long-K pair products read each operand block many times: grouped order;
  // short-K trailing updates: every position a tile, by columns
  auto tp_next = [](int t, int nrb_, int ncb_, int &rbl, int &cbl) {
    if constexpr (MAPPED) {
      return tp_tile_grouped(t, nrb_, ncb_, rbl, cbl);
    } else {
      tp_tile(t, nrb_, ncb_, rbl, cbl);
      return true;
    }
  };
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  if (halt && *(volatile const int *)halt) return;  // queued behind a fast panel that stopped early
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tp_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t *full = bar, *empty = bar + TP_STAGES, *accf = bar + 2 * TP_STAGES, *acce = accf + 2;
  if (warp == 1) t5::tmem_alloc(t5::smem_u32(&s_tmem), 2 * t5::TN);
  if (tid == 0) {
    s_abort = 0;
    for (int s = 0; s < TP_STAGES; ++s) {
      t5::mbar_init(t5::smem_u32(&full[s]), 1);
      t5::mbar_init(t5::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      t5::mbar_init(t5::smem_u32(&accf[b]), 1);
      t5::mbar_init(t5::smem_u32(&acce[b]), (TP_THREADS - 64) / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  t5::fence_before();
  __syncthreads();
  t5::fence_after();
  const uint32_t tmem = s_tmem;
  volatile int *abort = &s_abort;
  const int G = (int)gridDim.x;
  if (warp == 0) {
    if (lane == 0) {
      // producer: both operand blocks of every K chunk, in tile order
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntile && ok; t += G) {
        int rbl, cbl;
        if (!tp_next(t, nrb, ncb, rbl, cbl)) continue;
        const unsigned char *a = pack_a + (size_t)(blk0 + rbl) * nkc_stride * PK_BLOCK;
        const unsigned char *b = pack_b + (size_t)(blk0 + cbl) * nkc_stride * PK_BLOCK;
        for (int kc = kc0; kc < kc1; ++kc, ++it) {
          const int s = (int)(it % TP_STAGES);
          const uint32_t use = it / TP_STAGES;
          if (use > 0 && !tp_wait(t5::smem_u32(&empty[s]), (use - 1) & 1, abort, status)) {
            ok = false;
            break;
          }
          const uint32_t dst = t5::smem_u32(base + (size_t)s * t5::STAGE_BYTES);
          const uint32_t fb = t5::smem_u32(&full[s]);
          t5::mbar_arrive_expect_tx(fb, 2 * PK_BLOCK);
          t5::bulk_g2s(dst, a + (size_t)kc * PK_BLOCK, PK_BLOCK, fb);
          t5::bulk_g2s(dst + PK_BLOCK, b + (size_t)kc * PK_BLOCK, PK_BLOCK, fb);
        }
      }
      // copies still in flight land before the CTA leaves
      for (int s = 0; s < TP_STAGES; ++s)
        if (it > (uint32_t)s) t5::mbar_wait(t5::smem_u32(&full[s]), ((it - 1 - s) / TP_STAGES) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issue: 3 split products per 32-byte K step (8 TF32 or 16 BF16 entries)
      constexpr uint32_t IDESC = BF ? t5::idesc_bf16(t5::TM, t5::TN) : t5::idesc_tf32(t5::TM, t5::TN);
      auto mma = [](uint32_t d_, uint64_t a_, uint64_t b_, uint32_t acc_) {
        if constexpr (BF) t5::mma_bf16(d_, a_, b_, IDESC, acc_);
        else t5::mma_tf32(d_, a_, b_, IDESC, acc_);
      };
      uint32_t it = 0, last_bar = 0, last_par = 0;
      bool ok = true, any = false;
      int i = 0;
      for (int t = blockIdx.x; t < ntile && ok; t += G) {
        int rbl, cbl;
        if (!tp_next(t, nrb, ncb, rbl, cbl)) continue;
        const int buf = i & 1;
        const uint32_t u = (uint32_t)i >> 1;
        if (u > 0 && !tp_wait(t5::smem_u32(&acce[buf]), (u - 1) & 1, abort, status)) break;
        t5::fence_after();
        const uint32_t d = tmem + (uint32_t)(buf * t5::TN);
        for (int kc = kc0; kc < kc1; ++kc, ++it) {
          const int s = (int)(it % TP_STAGES);
          const uint32_t use = it / TP_STAGES;
          if (!tp_wait(t5::smem_u32(&full[s]), use & 1, abort, status)) {
            ok = false;
            break;
          }
          t5::fence_after();
          const uint32_t a_hi = t5::smem_u32(base + (size_t)s * t5::STAGE_BYTES), a_lo = a_hi + t5::OPND_BYTES;
          const uint32_t b_hi = a_hi + 2 * t5::OPND_BYTES, b_lo = a_hi + 3 * t5::OPND_BYTES;
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t off = ks * 32;
            const uint32_t acc0 = (kc > kc0 || ks > 0) ? 1u : 0u;
            mma(d, t5::desc_sw128(a_lo + off), t5::desc_sw128(b_hi + off), acc0);
            mma(d, t5::desc_sw128(a_hi + off), t5::desc_sw128(b_lo + off), 1u);
            mma(d, t5::desc_sw128(a_hi + off), t5::desc_sw128(b_hi + off), 1u);
          }
          t5::mma_commit(t5::smem_u32(&empty[s]));
          last_bar = t5::smem_u32(&empty[s]);
          last_par = use & 1;
          any = true;
        }
        if (ok) t5::mma_commit(t5::smem_u32(&accf[buf]));
        ++i;
      }
      // MMAs still running finish before the TMEM is released
      if (any) t5::mbar_wait(last_bar, last_par);
    }
  } else {
    if constexpr (MAPPED) {
      // epilogue: thread = TMEM lane = tile row, 64 of the tile's columns
      const int q = warp & 3, r = q * 32 + lane, cofs = ((warp - 2) >> 2) * 64;
      int i = 0;
      for (int t = blockIdx.x; t < ntile; t += G) {
        int rbl, cbl;
        if (!tp_next(t, nrb, ncb, rbl, cbl)) continue;
        const int buf = i & 1;
        const uint32_t u = (uint32_t)i >> 1;
        const int gi = (blk0 + rbl) * t5::TM + r, gj0 = (blk0 + cbl) * t5::TN + cofs;
        const int pr = gi < mrows ? prow[gi] : -1;
        const int jhi = pr >= 0 ? min(64, min(ncols - gj0, gi - gj0 + 1)) : 0;  // columns gj0 + [0, jhi)
        int okw = 0;
        if (lane == 0) okw = tp_wait(t5::smem_u32(&accf[buf]), u & 1, abort, status) ? 1 : 0;
        if (!__shfl_sync(0xffffffffu, okw, 0)) break;
        t5::fence_after();
#pragma unroll 1
        for (int g = 0; g < 2; ++g) {
          uint32_t v[32];
          t5::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * t5::TN + cofs + g * 32), v);
          float cur[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int jj = g * 32 + j;
            const int pc = jj < jhi ? __ldg(pcol + gj0 + jj) : -1;
            cur[j] = pc >= 0 ? S[(size_t)pc * nrow + pr] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int jj = g * 32 + j;
            const int pc = jj < jhi ? __ldg(pcol + gj0 + jj) : -1;
            if (pc >= 0) S[(size_t)pc * nrow + pr] = cur[j] - __uint_as_float(v[j]);
          }
        }
        t5::fence_before();
        __syncwarp();
        if (lane == 0) t5::mbar_arrive(t5::smem_u32(&acce[buf]));
        ++i;
      }
    } else {
      // epilogue: thread = TMEM lane = tile row, 64 of the tile's columns
      const int q = warp & 3, r = q * 32 + lane, cofs = ((warp - 2) >> 2) * 64;
      int i = 0;
      for (int t = blockIdx.x; t < ntile; t += G) {
        int rbl, cbl;
        if (!tp_next(t, nrb, ncb, rbl, cbl)) continue;
        const int buf = i & 1;
        const uint32_t u = (uint32_t)i >> 1;
        const int gr = (blk0 + rbl) * t5::TM + r, gc0 = (blk0 + cbl) * t5::TN + cofs;
        // columns gc0 + [jlo, jhi) of row gr are in the update (gc >= cb,
        // gc < ce, gc <= gr); their current values are loaded first, so that
        // the latency overlaps the tile's MMAs
        const int jlo = max(0, cb - gc0);
        const int jhi = gr < nrow ? min(64, min(ce - gc0, gr - gc0 + 1)) : 0;
        float *row = S + gr + (size_t)gc0 * nrow;
        const size_t ld = (size_t)nrow;
        float cur[64];
        {
          const float *pp = row;
#pragma unroll
          for (int j = 0; j < 64; ++j) {
            cur[j] = (j >= jlo && j < jhi) ? __ldcs(pp) : 0.f;
            pp += ld;
          }
        }
        // one lane waits, so that the whole warp leaves or goes on together
        int okw = 0;
        if (lane == 0) okw = tp_wait(t5::smem_u32(&accf[buf]), u & 1, abort, status) ? 1 : 0;
        if (!__shfl_sync(0xffffffffu, okw, 0)) break;
        t5::fence_after();
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          uint32_t v[32];
          t5::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * t5::TN + cofs + g * 32), v);
          float *pp = row + (size_t)(g * 32) * ld;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int jj = g * 32 + j;
            if (jj >= jlo && jj < jhi) *pp = cur[jj] - __uint_as_float(v[j]);
            pp += ld;
          }
        }
        t5::fence_before();
        __syncwarp();
        if (lane == 0) t5::mbar_arrive(t5::smem_u32(&acce[buf]));
        ++i;
      }
    }
  }
  t5::fence_before();
  __syncthreads();
  if (warp == 1) {
    t5::fence_after();
    t5::tmem_dealloc(tmem, 2 * t5::TN);
  }
}

template <class T> __global__ void k_wide_init_perm(int *perm, int w) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < w; m += gridDim.x * blockDim.x) perm[m] = m;
}

template <class T> __global__ void k_wide_zero_upper(T *S, int nrow, int w) {
  // entries above the diagonal of the diagonal block stay 0
  for (int c = blockIdx.x; c < w; c += gridDim.x)
    for (int r = threadIdx.x; r < c; r += blockDim.x) S[r + (size_t)c * nrow] = T(0);
}

}  // namespace

// Panel / trailing-update sequence of one wide supernode: values S (nrow x
// w, column-major), D and E (diagonal, 2x2 sub-diagonals), in-block pivot
// order perm; scratch Wb (nrow x (nb+2)) and ctl.  P, when given, receives the
// launch count and the per-class timings.
template <class T>
static int run_wide(T *S, int nrow, int w, T *Dd, T *De, int *perm, T *Wb, WideCtl *ctl, int *status,
                    cudaStream_t st, int num_sms, int nb, int *pivoted, Plan *P, int depth) {
  if (nb > WP_NB || nb < 1) return NQG_ERR_ARG;
  k_wide_init_perm<T><<<(w + 255) / 256, 256, 0, st>>>(perm, w);
  if (P) P->nlaunch++;
  if (cudaMemsetAsync(ctl, 0, offsetof(WideCtl, spin_limit), st) != cudaSuccess) return NQG_ERR_CUDA;
  const size_t smem = (size_t)(WP_NB + 2) * WP_THREADS * sizeof(T);
  // per call: the attribute belongs to the current device
  if (cudaFuncSetAttribute(k_wide_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return NQG_ERR_CUDA;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_wide_panel<T>, WP_THREADS, smem) != cudaSuccess)
    return NQG_ERR_CUDA;
  const int maxG = std::max(1, std::min(occ * num_sms, 1024));
  // FP32 trailing updates: the persistent tcgen05 kernel on packed split
  // operands (BF16; NASOQ_GB300_SPLIT=tf32 for TF32) by default;
  // NASOQ_GB300_TRAILING=mma selects the mma.sync split-TF32 kernel and
  // =simt the CUDA-core kernel
  // NASOQ_GB300_TRAILING=tile keeps the tcgen05 updates on one CTA per tile
  // with operands split while they are loaded, instead of the persistent
  // kernel on packed operands
  const char *te = std::getenv("NASOQ_GB300_TRAILING");
  const int trail = !te ? 2 : std::string(te) == "simt" ? 0 : std::string(te) == "mma" ? 1 : 2;
  const bool tile_only = te && std::string(te) == "tile";
  // packed split operands: row blocks of A (L rows) then of B (W rows),
  // nkc_stride chunks each (every pending panel starts on a new chunk)
  unsigned char *pack_a = (sizeof(T) == 4 && trail == 2 && !tile_only && P) ? P->d_wide_pack : nullptr;
  const bool bf = pk_bf16();
  const int kchunk = pk_chunk(bf);
  const int nch_panel = (nb + 1 + kchunk - 1) / kchunk;
  const int nkc_stride = (std::max(depth, 1) + 1) * nch_panel;  // room for depth + 1 panels
  const int nrb_all = (nrow + t5::TM - 1) / t5::TM, ncb_all = (w + t5::TN - 1) / t5::TN;
  unsigned char *pack_b = pack_a ? pack_a + (size_t)nrb_all * nkc_stride * PK_BLOCK : nullptr;
  if (pack_a && cudaFuncSetAttribute(bf ? k_tc_persistent<false, true> : k_tc_persistent<false, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tp_smem_bytes()) != cudaSuccess)
    return NQG_ERR_CUDA;
  if (sizeof(T) == 4 && trail == 1 &&
      cudaFuncSetAttribute(k_wide_trailing_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) !=
          cudaSuccess)
    return NQG_ERR_CUDA;
  if (sizeof(T) == 4 && trail == 2 &&
      cudaFuncSetAttribute(k_wide_trailing_t5, cudaFuncAttributeMaxDynamicSharedMemorySize, t5::smem_bytes(1)) !=
          cudaSuccess)
    return NQG_ERR_CUDA;
  // FP32: fast panels (no pivot search) until a column needs one; the
  // general kernel then factors one panel from that column.
  // NASOQ_GB300_PANEL=general keeps every panel on the general kernel.
  // NASOQ_GB300_PANEL=general keeps every panel on the general kernel;
  // =group keeps fast panels on the grouped kernel (four columns per
  // exchange) instead of the block-first one (one exchange per panel).
  const char *pe = std::getenv("NASOQ_GB300_PANEL");
  const bool fast_enabled = sizeof(T) == 4 && !(pe && std::string(pe) == "general");
  const bool blk_enabled = fast_enabled && !(pe && std::string(pe) == "group");
  const size_t fsmem = fast_panel_smem(nb);
  int maxG_fast = 0, maxG_blk = 0;
  if (fast_enabled) {
    if (cudaFuncSetAttribute(k_wide_panel_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem) !=
        cudaSuccess)
      return NQG_ERR_CUDA;
    int occf = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occf, k_wide_panel_fast, FP_THREADS, fsmem) != cudaSuccess)
      return NQG_ERR_CUDA;
    maxG_fast = std::min(std::max(occf, 0) * num_sms, 1024);
  }
  if (blk_enabled) {
    if (cudaFuncSetAttribute(k_wide_panel_blk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fast_blk_smem()) != cudaSuccess)
      return NQG_ERR_CUDA;
    int occb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occb, k_wide_panel_blk, FB_THREADS, fast_blk_smem()) !=
        cudaSuccess)
      return NQG_ERR_CUDA;
    maxG_blk = std::min(std::max(occb, 0) * num_sms, FB_MAXG);
  }
  // exchange words of the block-first kernel: seq per launch; the grouped
  // kernel leaves words of its own format behind (cleared before the next
  // block-first launch)
  unsigned blk_seq = 0;
  bool mslot_dirty = false;
  // width of general panels that follow a fast panel's stop (FP32 fast-panel
  // path: 8 columns, NASOQ_GB300_PIVOT_NB overrides, 2 .. nb): the pivots of
  // the KKT systems come singly or in 2 x 2 blocks, so the fast kernel takes
  // over again right after them
  int pivot_nb = fast_enabled ? std::min(nb, 8) : nb;
  if (const char *e = std::getenv("NASOQ_GB300_PIVOT_NB"))
    if (fast_enabled) pivot_nb = std::min(nb, std::max(2, std::atoi(e)));
  // where pivots are dense (a fast panel stops again within nb / 4 columns)
  // the general panels double in width, up to nb, so that fewer of them --
  // each flushes the pending updates -- are needed; back to pivot_nb after a
  // fast panel that stops late or not at all
  int gen_w = pivot_nb;
  auto after_fast = [&](bool stopped, int kept) {
    gen_w = !stopped || kept >= nb / 4 ? pivot_nb : std::min(nb, 2 * gen_w);
  };
  bool use_general = false;  // the next panel starts at a column that needs a pivot search
  // Delayed trailing updates (FP32 tcgen05 path): up to `depth` consecutive
  // panels are pending, their W columns side by side in Wb, and one update of
  // K = their total width flushes them to the columns beyond the frontier F.
  // Invariant: columns < F carry the update of every pending panel, columns
  // >= F of none.  Before a panel, the band from F to its last possible
  // column (k0 + nb, or k0 + nb + 1 for a final 2x2 of the general kernel) is
  // brought up to date; after it,
  // the panel's own update covers [k1, F).  A panel on the general kernel may
  // interchange rows and columns anywhere in the trailing block, so every
  // pending update is flushed before it.
  //
  // Speculation (FP32 tcgen05 path): fast panels are queued assuming they
  // factor all their columns, up to SPEC_MAX per host synchronisation, with
  // the updates that follow from that assumption.  A fast panel that stops
  // early sets ctl->halt and every kernel queued after it returns untouched;
  // at the next synchronisation the host restores the state it saved before
  // that panel's updates and replays them with the real column count.
  const bool delayed = sizeof(T) == 4 && trail == 2 && depth > 1;
  const bool spec_ok = fast_enabled && trail == 2;
  constexpr int SPEC_MAX = 16;
  struct State {
    int k0, F, pend_k0, pend_K, npend, pend_C;  // pend_C: packed chunks of the pending panels
  };
  struct Spec {
    State st;  // state after the panel's band update, before the panel
    int kb, woff;
    size_t prof_mark;  // measurement records after the panel's own
  };
  State cs{0, 0, 0, 0, 0, 0};
  std::vector<Spec> specs;
  int spec_limit = SPEC_MAX;  // batch size: 1 after a rewind, doubling after each clean batch
  const int *halt = &ctl->halt;
  // chunks of a panel of kb columns in the pack buffer
  auto nch = [&](int kb) { return (kb + kchunk - 1) / kchunk; };
  // split blocks of a finished panel (columns k0 .. k0+kb-1, W at column
  // woff of Wb) into chunks kcs .. of the pack buffer, rows from the block
  // holding k0 + kb on (the rows every later update of it touches)
  auto pack_panel = [&](int k0, int kb, int woff, int kcs) -> int {
    const int k1 = k0 + kb;
    if (!pack_a || k1 >= w || kb <= 0) return NQG_OK;
    cudaEvent_t e1 = P ? P->prof_begin() : nullptr;
    const int rb_first = k1 / t5::TM;
    int ld = nrow;
    auto pk = bf ? k_pack_split<true> : k_pack_split<false>;
    pk<<<dim3(nrb_all - rb_first, nch(kb)), 256, 0, st>>>(reinterpret_cast<const float *>(S) + (size_t)k0 * nrow, ld,
                                                          nrow, kb, pack_a, nkc_stride, kcs, rb_first, halt);
    pk<<<dim3(ncb_all - rb_first, nch(kb)), 256, 0, st>>>(reinterpret_cast<const float *>(Wb) + (size_t)woff * nrow,
                                                          ld, w, kb, pack_b, nkc_stride, kcs, rb_first, halt);
    if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
    if (P) {
      P->nlaunch += 2;
      // FP32 read once, hi + lo written
      const double bytes = (double)kb * ((nrow - rb_first * t5::TM) + (w - rb_first * t5::TM)) * (bf ? 8.0 : 12.0);
      P->prof_end(NQG_K_PACK, e1, 0.0, bytes);
    }
    return NQG_OK;
  };
  // S[cb.., cb..ce) -= L(:, kL .. kL+K) W(:, woff ..)^T (lower part); with
  // packed operands the same product from chunks kca .. kcb-1
  auto apply = [&](int kL, int K, int woff, int kca, int kcb, int cb, int ce) -> int {
    if (ce <= cb || K <= 0) return NQG_OK;
    cudaEvent_t e1 = P ? P->prof_begin() : nullptr;
    if (pack_a) {
      const int blk0 = cb / t5::TM;
      const int nrb = nrb_all - blk0, ncb = (ce + t5::TN - 1) / t5::TN - blk0;
      const int ntile = ncb * nrb - ncb * (ncb - 1) / 2;
      const int G = std::max(1, std::min(ntile, num_sms));
      float *Sf = reinterpret_cast<float *>(S);
      auto kt = bf ? k_tc_persistent<false, true> : k_tc_persistent<false, false>;
      kt<<<G, TP_THREADS, tp_smem_bytes(), st>>>(Sf, nrow, cb, ce, pack_a, pack_b, nkc_stride, kca, kcb, blk0, nrb,
                                                 ncb, ntile, halt, status, nullptr, nullptr, 0, 0);
    } else {
      const int tm = (nrow - cb + t5::TM - 1) / t5::TM, tn = (ce - cb + t5::TN - 1) / t5::TN;
      k_wide_trailing_t5<<<tm * tn, t5::THREADS, t5::smem_bytes(1), st>>>(
          reinterpret_cast<float *>(S), nrow, kL, K, cb, ce,
          reinterpret_cast<const float *>(Wb) + (size_t)woff * nrow, nrow, tn, halt, status);
    }
    if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
    if (P) {
      P->nlaunch++;
      const double cols = ce - cb;
      const double entries = cols * (nrow - cb) - cols * (cols - 1) / 2.0;
      P->prof_end(NQG_K_WIDE_TRAILING, e1, 2.0 * K * entries, 0.0);
    }
    return NQG_OK;
  };
  // band update before a panel at s.k0 (flushing everything before a general one)
  auto pre = [&](State &s, bool general, int kb_want) -> int {
    if (!delayed) return NQG_OK;
    int rc;
    if (general && s.npend > 0) {
      if ((rc = apply(s.pend_k0, s.pend_K, 0, 0, s.pend_C, s.F, w))) return rc;
      s.npend = 0;
      s.pend_K = 0;
      s.pend_C = 0;
      s.F = s.k0;
    }
    // a general panel may end with a 2x2 pivot one column past nb; a fast
    // panel never goes past nb, so its band stops at k0 + nb and a complete
    // fast panel leaves no remainder of its own update to apply
    const int bend = std::min(w, s.k0 + kb_want + (general ? 1 : 0));
    if (s.npend > 0 && s.F < bend && (rc = apply(s.pend_k0, s.pend_K, 0, 0, s.pend_C, s.F, bend))) return rc;
    s.F = std::max(s.F, bend);
    return NQG_OK;
  };
  // updates after a panel of kb columns at s.k0 whose W starts at column woff
  auto post = [&](State &s, int kb, int woff, bool packed) -> int {
    const int k0 = s.k0, k1 = k0 + kb;
    int rc;
    if (delayed) {
      if (!packed && (rc = pack_panel(k0, kb, woff, s.pend_C))) return rc;
      if (k1 < s.F && (rc = apply(k0, kb, woff, s.pend_C, s.pend_C + nch(kb), k1, s.F))) return rc;
      if (s.npend == 0) s.pend_k0 = k0;
      s.pend_K += kb;
      s.pend_C += nch(kb);
      ++s.npend;
      // flush once depth * nb columns are pending (narrow panels after pivot
      // searches do not count as whole panels), or before the buffers (room
      // for depth + 1 panels of nb + 1 columns) could overflow
      if (s.pend_K >= depth * nb || s.pend_C + nch(nb + 1) > nkc_stride ||
          s.pend_K + nb + 1 > (depth + 1) * (nb + 1) || k1 >= w) {
        if ((rc = apply(s.pend_k0, s.pend_K, 0, 0, s.pend_C, s.F, w))) return rc;
        s.npend = 0;
        s.pend_K = 0;
        s.pend_C = 0;
        s.F = k1;
      }
    } else if (k1 < w && pack_a) {
      if ((!packed && (rc = pack_panel(k0, kb, 0, 0))) || (rc = apply(k0, kb, 0, 0, nch(kb), k1, w))) return rc;
    } else if (k1 < w) {
      cudaEvent_t e1 = P ? P->prof_begin() : nullptr;
      if (sizeof(T) == 4 && trail == 2) {
        int tm = (nrow - k1 + t5::TM - 1) / t5::TM, tn = (w - k1 + t5::TN - 1) / t5::TN;
        k_wide_trailing_t5<<<tm * tn, t5::THREADS, t5::smem_bytes(1), st>>>(
            reinterpret_cast<float *>(S), nrow, k0, kb, k1, w, reinterpret_cast<const float *>(Wb), nrow, tn, halt,
            status);
      } else if (sizeof(T) == 4 && trail == 1) {
        int tm = (nrow - k1 + TC_BM - 1) / TC_BM, tn = (w - k1 + TC_BN - 1) / TC_BN;
        k_wide_trailing_tc<<<tm * tn, 256, TC_SMEM, st>>>(reinterpret_cast<float *>(S), nrow, w, k0, kb,
                                                          reinterpret_cast<const float *>(Wb), nrow, tn);
      } else if (sizeof(T) == 4) {
        constexpr int BM = 128, BN = 128;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 8, 8><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      } else {
        constexpr int BM = 64, BN = 64;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 4, 4><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      }
      if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
      if (P) {
        P->nlaunch++;
        // useful multiply-adds: kb per entry of the lower trapezoid rows [k1,nrow) x cols [k1,w)
        const double cols = w - k1;
        const double entries = cols * (nrow - k1) - cols * (cols - 1) / 2.0;
        P->prof_end(NQG_K_WIDE_TRAILING, e1, 2.0 * kb * entries, 0.0);
      }
    }
    s.k0 = k1;
    return NQG_OK;
  };
  auto panel_flops = [&](int k0, int kb) {
    double fl = 0;  // column GEMVs (2 * rows * j) and the L column scaling
    for (int jj = 0; jj < kb; ++jj) fl += 2.0 * (nrow - (k0 + jj)) * (jj + 1);
    return fl;
  };
  // packed: set when the block-first kernel packs the panel's operands itself
  // (chunks from kcs on)
  auto launch_fast = [&](int k0, int kb_want, T *Wp, int slot, int kcs, bool &packed) -> int {
    packed = false;
    const int rows_out = nrow - k0 - kb_want;
    int ldw = nrow;
    float *Sf = reinterpret_cast<float *>(S), *Wf = reinterpret_cast<float *>(Wp);
    float *Df = reinterpret_cast<float *>(Dd), *Ef = reinterpret_cast<float *>(De);
    const int Gb = std::max(1, (rows_out + FB_THREADS - 1) / FB_THREADS);
    if (blk_enabled && Gb <= maxG_blk) {
      if (mslot_dirty) {
        if (cudaMemsetAsync(&ctl->mslot[0][0][0], 0, sizeof(ctl->mslot), st) != cudaSuccess) return NQG_ERR_CUDA;
        mslot_dirty = false;
      }
      if (++blk_seq == 0) blk_seq = 1;
      unsigned seq = blk_seq;
      unsigned char *pa = k0 + kb_want < w ? pack_a : nullptr, *pb = pack_b;
      int nkcs = nkc_stride, pkbf = bf ? 1 : 0;
      void *args[] = {&Sf, &nrow, &w, &k0, &kb_want, &Wf, &ldw, &Df, &Ef, &ctl, &slot, &seq, &status, &pa, &pb,
                      &nkcs, &kcs, &pkbf};
      cudaEvent_t e0 = P ? P->prof_begin() : nullptr;
      if (cudaLaunchCooperativeKernel((void *)k_wide_panel_blk, dim3(Gb), dim3(FB_THREADS), args, fast_blk_smem(),
                                      st) != cudaSuccess)
        return NQG_ERR_CUDA;
      if (P) {
        P->nlaunch++;
        P->prof_end(NQG_K_WIDE_PANEL, e0, panel_flops(k0, kb_want), 0.0);
      }
      packed = pa != nullptr;
      return NQG_OK;
    }
    const int G = std::max(1, std::min(maxG_fast, (rows_out + FP_THREADS - 1) / FP_THREADS));
    void *args[] = {&Sf, &nrow, &w, &k0, &kb_want, &Wf, &ldw, &Df, &Ef, &ctl, &slot, &status};
    if (cudaMemsetAsync(&ctl->mslot[0][0][0], 0, sizeof(ctl->mslot), st) != cudaSuccess) return NQG_ERR_CUDA;
    mslot_dirty = true;
    cudaEvent_t e0 = P ? P->prof_begin() : nullptr;
    if (cudaLaunchCooperativeKernel((void *)k_wide_panel_fast, dim3(G), dim3(FP_THREADS), args, fsmem, st) !=
        cudaSuccess)
      return NQG_ERR_CUDA;
    if (P) {
      P->nlaunch++;
      P->prof_end(NQG_K_WIDE_PANEL, e0, panel_flops(k0, kb_want), 0.0);
    }
    return NQG_OK;
  };
  // synchronise with a speculative batch; replay from its first short panel
  auto resolve = [&]() -> int {
    if (specs.empty()) return NQG_OK;
    const int n = (int)specs.size();
    int kbs[SPEC_MAX] = {}, abort = 0;
    if (cudaMemcpyAsync(kbs, ctl->kb_log, n * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&abort, &ctl->abort, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return NQG_ERR_CUDA;
    if (abort) return NQG_ERR_TIMEOUT;
    int i = 0;
    while (i < n && kbs[i] == specs[i].kb) ++i;
    if (i < n) {
      if (cudaMemsetAsync(&ctl->halt, 0, sizeof(int), st) != cudaSuccess) return NQG_ERR_CUDA;
      // everything queued after the short panel returned without work
      if (P) P->prof_void_from(specs[i].prof_mark);
      cs = specs[i].st;
      if (kbs[i] > 0) {
        // a short panel did not pack the rows of its diagonal block below its
        // last column: pack_panel does it all again
        int rc = post(cs, kbs[i], specs[i].woff, false);
        if (rc) return rc;
      }
      use_general = true;  // the column after the short panel needs a pivot search
      spec_limit = 1;
      after_fast(true, kbs[i]);
    } else {
      spec_limit = std::min(SPEC_MAX, 2 * spec_limit);
      after_fast(false, 0);
    }
    specs.clear();
    if (P) P->prof_hold = false;
    return NQG_OK;
  };
  while (cs.k0 < w) {
    // a panel on the general kernel (after a fast panel stopped at a column
    // that needs a pivot search) is at most gen_w columns wide, so that the
    // fast kernel takes over again soon after the pivots
    const int kb_want = std::min(use_general ? gen_w : nb, w - cs.k0);
    const bool fast = fast_enabled && !use_general && nrow - cs.k0 - kb_want <= maxG_fast * FP_THREADS;
    if (fast && spec_ok) {
      int rc = pre(cs, false, kb_want);
      if (rc) return rc;
      const int woff = delayed ? cs.pend_K : 0;
      bool packed = false;
      if ((rc = launch_fast(cs.k0, kb_want, Wb + (size_t)woff * nrow, (int)specs.size(), delayed ? cs.pend_C : 0,
                            packed)))
        return rc;
      if (P) P->prof_hold = true;
      specs.push_back(Spec{cs, kb_want, woff, P ? P->prof_mark() : 0});
      if ((rc = post(cs, kb_want, woff, packed))) return rc;
      if (((int)specs.size() >= spec_limit || cs.k0 >= w) && (rc = resolve())) return rc;
      continue;
    }
    if (!specs.empty()) {
      int rc = resolve();
      if (rc) return rc;
      continue;  // the state may have been rewound
    }
    int rc = pre(cs, !fast, kb_want);
    if (rc) return rc;
    const int woff = delayed ? cs.pend_K : 0;  // this panel's W columns
    T *Wp = Wb + (size_t)woff * nrow;
    int kb = 0, abort = 0, stop = 0, ldw = nrow, kbw = kb_want, k0 = cs.k0;
    bool packed = false;
    if (fast) {
      if ((rc = launch_fast(k0, kb_want, Wp, -1, delayed ? cs.pend_C : 0, packed))) return rc;
    } else {
      if (cudaMemsetAsync(&ctl->pslot[0][0], 0, sizeof(ctl->pslot), st) != cudaSuccess) return NQG_ERR_CUDA;
      cudaEvent_t e0 = P ? P->prof_begin() : nullptr;
      // one row per thread where the grid allows it
      const int rows_left = nrow - k0;
      const int G = std::max(1, std::min(maxG, (rows_left + WP_THREADS - 1) / WP_THREADS));
      void *args[] = {&S, &nrow, &w, &k0, &kbw, &Wp, &ldw, &Dd, &De, &perm, &ctl, &status};
      if (cudaLaunchCooperativeKernel((void *)k_wide_panel<T>, dim3(G), dim3(WP_THREADS), args, smem, st) !=
          cudaSuccess)
        return NQG_ERR_CUDA;
      if (P) {
        P->nlaunch++;
        P->prof_end(NQG_K_WIDE_PIVOT, e0, panel_flops(k0, kb_want), 0.0);
      }
    }
    if (cudaMemcpyAsync(&kb, &ctl->kb, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&abort, &ctl->abort, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&stop, &ctl->stop, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return NQG_ERR_CUDA;
    if (abort) return NQG_ERR_TIMEOUT;
    if (fast) {
      use_general = stop != 0;
      after_fast(use_general, kb);
      if (kb <= 0) {
        if (!use_general) return NQG_ERR_TIMEOUT;
        continue;  // the first column already needs the general kernel
      }
    } else {
      use_general = false;
      if (kb <= 0) return NQG_ERR_TIMEOUT;
    }
    if ((rc = post(cs, kb, woff, packed && kb == kb_want))) return rc;
  }
  k_wide_zero_upper<T><<<std::min(w, 1024), 128, 0, st>>>(S, nrow, w);
  if (P) P->nlaunch++;
  if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
  int piv = 0;
  if (cudaMemcpyAsync(&piv, &ctl->pivoted, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return NQG_ERR_CUDA;
  if (pivoted) *pivoted = piv;
  return NQG_OK;
}

// Host driver for one wide supernode s of a plan.
template <class T>
int factor_wide(Plan &P, int s, T *L, T *Dg, int nb, T *Wb, WideCtl *ctl, int num_sms) {
  const int c0 = P.sym.super[s], w = P.sym.super[s + 1] - c0;
  const int nrow = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
  int piv = 0;
  int rc = run_wide<T>(L + P.sym.lpx[s], nrow, w, Dg + c0, Dg + P.n + c0, P.d_locperm + c0, Wb, ctl, P.d_status,
                       P.stream, num_sms, nb, &piv, &P, P.wide_depth);
  if (rc == NQG_ERR_CUDA) {
    cudaError_t e = cudaGetLastError();
    P.last_error = cudaGetErrorString(e);
  }
  if (rc) return rc;
  uint8_t pv = piv ? 1 : 0;
  NQG_CUDA(cudaMemcpyAsync(P.d_pivoted + s, &pv, 1, cudaMemcpyHostToDevice, P.stream));
  NQG_CUDA(cudaStreamSynchronize(P.stream));
  return NQG_OK;
}

// Schur update of target s by descendant pair q as one persistent launch:
// target positions, packed (L D) rows and L rows of the pair, then the
// tcgen05 product subtracted in place (the pair's tiles are disjoint, and no
// other update of the target runs at the same time).
int update_pair_persistent(Plan &P, int s, int q, float *L, const float *Dg) {
  const int d = P.pair_d[q], lb = P.pair_lb[q], ub = P.pair_ub[q];
  const int c0 = P.sym.super[d], wd = P.sym.super[d + 1] - c0;
  const int nrd = (int)(P.sym.lpi[d + 1] - P.sym.lpi[d]);
  const int cs0 = P.sym.super[s], ws = P.sym.super[s + 1] - cs0;
  const int nrs = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
  const int m = nrd - lb, nc = ub - lb + 1;
  if (m <= 0 || nc <= 0 || wd <= 0) return NQG_OK;
  const bool bf = pk_bf16();
  const int nkc = (wd + pk_chunk(bf) - 1) / pk_chunk(bf), nrb = (m + t5::TM - 1) / t5::TM,
            ncb = (nc + t5::TN - 1) / t5::TN;
  unsigned char *pa = P.d_wide_pack, *pb = pa + (size_t)nrb * nkc * PK_BLOCK;
  int *prow = P.d_pers_map, *pcol = prow + m;
  if (!pa || !prow) return NQG_ERR_ARG;
  cudaStream_t st = P.stream;
  auto kt = bf ? k_tc_persistent<true, true> : k_tc_persistent<true, false>;
  if (cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tp_smem_bytes()) != cudaSuccess)
    return NQG_ERR_CUDA;
  cudaEvent_t ep = P.prof_begin();
  k_pair_map<<<std::min((m + 255) / 256, 1024), 256, 0, st>>>(P.d_ls + P.sym.lpi[d] + lb, m, nc,
                                                              P.d_ls + P.sym.lpi[s], nrs, cs0, ws, prow, pcol,
                                                              P.d_status);
  const float *Ld = L + P.sym.lpx[d] + lb;
  (bf ? k_pack_ld<true> : k_pack_ld<false>)<<<dim3(nrb, nkc), 256, 0, st>>>(Ld, nrd, m, wd, Dg + c0, Dg + P.n + c0,
                                                                           pa, nkc);
  (bf ? k_pack_split<true> : k_pack_split<false>)<<<dim3(ncb, nkc), 256, 0, st>>>(Ld, nrd, nc, wd, pb, nkc, 0, 0,
                                                                                 nullptr);
  P.prof_end(NQG_K_PACK, ep, 0.0, (double)(m + nc) * wd * (bf ? 8.0 : 12.0));
  cudaEvent_t e0 = P.prof_begin();
  const int ntile = ncb * nrb - ncb * (ncb - 1) / 2;
  const int G = std::max(1, std::min(ntile, P.num_sms));
  const int nflat = (int)tp_flat_count(nrb, ncb);
  kt<<<G, TP_THREADS, tp_smem_bytes(), st>>>(L + P.sym.lpx[s], nrs, 0, 0, pa, pb, nkc, 0, nkc, 0, nrb, ncb, nflat,
                                             nullptr, P.d_status, prow, pcol, m, nc);
  if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
  P.nlaunch += 4;
  P.prof_end(NQG_K_UPDATE, e0, P.pair_flops[q], 0.0);
  return NQG_OK;
}

size_t wide_ctl_bytes() { return sizeof(WideCtl); }
size_t wide_ctl_limit_offset() { return offsetof(WideCtl, spin_limit); }

// Same panel / trailing-update sequence as factor_wide, on caller-provided
// buffers (values S, D, E, perm) and caller-provided scratch (Wb, ctl,
// status); used by the allocation-free dense entry point.
template <class T>
int factor_wide_raw(T *S, int nrow, int w, T *Dd, T *De, int *perm, T *Wb, WideCtl *ctl, int *status,
                    cudaStream_t st, int num_sms, int nb, int *pivoted) {
  return run_wide<T>(S, nrow, w, Dd, De, perm, Wb, ctl, status, st, num_sms, nb, pivoted, nullptr, 1);
}

template int factor_wide_raw<double>(double *, int, int, double *, double *, int *, double *, WideCtl *, int *,
                                     cudaStream_t, int, int, int *);

template int factor_wide<float>(Plan &, int, float *, float *, int, float *, WideCtl *, int);
template int factor_wide<double>(Plan &, int, double *, double *, int, double *, WideCtl *, int);

}  // namespace nqg
