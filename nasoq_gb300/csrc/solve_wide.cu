// Forward and backward supernodal solves for one wide supernode, spread over
// the whole GPU (reference H2LeveledBlockedLsolve / LTsolve per supernode,
// src/triangularSolve/Triangular_BCSC.cpp:378-446, 534-600: dtrsm on the
// diagonal block + dgemv with the rows below).
//
// Both sweeps are persistent cooperative kernels without grid barriers.  The
// supernode's nrow x w panel is cut into 64 x 64 tiles.  Forward: work item q
// is block row q (64 rows of the diagonal block, then 64-row blocks of the rows
// below); it accumulates L(q, j) x_j over the column blocks j before it, each
// as soon as block j's ready flag carries this launch's epoch, then solves
// its 64 x 64 unit-lower diagonal tile in one warp and publishes x_q with a
// release store of its flag (rows below scatter L21 x into the ancestors'
// entries with atomics instead).  Backward: item j is column block j, taken
// from the last; it gathers L21^T x(rows below) without waiting, then
// L(i, j)^T x_i for i > j as those blocks become ready, and solves the
// transposed diagonal tile.  Each CTA takes its items in dependency order, and
// a cooperative launch keeps all CTAs resident, so every wait ends; each wait
// is still bounded (timeout -> ST_TIMEOUT and an abort flag the other CTAs
// see).  Matrix tiles do not depend on the flags, so the next tile's values
// are loaded before the wait for the current one.
#include <cuda_runtime.h>

#include <algorithm>

#include "coop.cuh"
#include "plan.hpp"

namespace nqg {

namespace {

constexpr int SW_THREADS = 256;
constexpr int TB = 64;                       // tile rows / columns
constexpr int CPT = TB / (SW_THREADS / TB);  // tile columns per thread (16)

// x_b := L11[b]^-1 x_b for a 64x64 unit lower block, one warp, lane i holds
// rows i and i+32; T11 is the block staged column-major in shared memory.
template <class V> __device__ void warp_trsv_lower(const V *T11, int m, V *xb) {
  const int lane = threadIdx.x & 31;
  V v0 = lane < m ? xb[lane] : V(0), v1 = lane + 32 < m ? xb[lane + 32] : V(0);
  for (int j = 0; j < m; ++j) {
    const V xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31);
    if (lane > j && lane < m) v0 -= T11[lane + j * TB] * xj;
    if (lane + 32 > j && lane + 32 < m) v1 -= T11[lane + 32 + j * TB] * xj;
  }
  if (lane < m) xb[lane] = v0;
  if (lane + 32 < m) xb[lane + 32] = v1;
}

// x_b := L11[b]^-T x_b (backward substitution with the transposed block).
template <class V> __device__ void warp_trsv_lower_t(const V *T11, int m, V *xb) {
  const int lane = threadIdx.x & 31;
  V v0 = lane < m ? xb[lane] : V(0), v1 = lane + 32 < m ? xb[lane + 32] : V(0);
  for (int i = m - 1; i > 0; --i) {
    const V xi = __shfl_sync(0xffffffffu, i < 32 ? v0 : v1, i & 31);
    // x_j -= L(i, j) x_i for j < i
    if (lane < i) v0 -= T11[i + lane * TB] * xi;
    if (lane + 32 < i) v1 -= T11[i + (lane + 32) * TB] * xi;
  }
  if (lane < m) xb[lane] = v0;
  if (lane + 32 < m) xb[lane + 32] = v1;
}

// FP32 sweeps solve a diagonal tile by a product with its inverse, and take
// the last link of the dependency chain -- the block solved just before --
// through one more precomputed product:
//   forward   x_q = T_q (b_q - sum_{j<q-1} L(q,j) x_j) - Mf_q x_{q-1},
//             Mf_q = T_q L(q,q-1);
//   backward  x_j = T_j^T (b_j - sum_{i>j+1} L(i,j)^T x_i - ...) - Mb_j x_{j+1},
//             Mb_j = T_j^T L(j+1,j)^T;
// with T = L_qq^-1, so that once x_{q-1} arrives one 64 x 64 product remains.
// Formed once per factorization for every diagonal tile (s, j) of the
// block-solved supernodes: T, Mf, Mb at tinv + (flagoff[s] + j) * 3 * TI (+ 0,
// TI, 2 TI), entry (k, c) at [c * (TB + 1) + k], zeros outside the blocks.
constexpr int TI = TB * (TB + 1);

// One CTA of TB threads per diagonal tile (items: the backward items, (s, q)
// for column block nbd(s) - 1 - q).  Thread c forms column c of T by forward
// substitution in registers (its entries above row c start at 0 and stay 0,
// so the unrolled recurrences need no predicate), then column c of Mf and of
// Mb from T in shared memory.
__global__ void __launch_bounds__(TB) k_tile_inverse(const int2 *items, const int *super, const int64_t *lpi,
                                                     const int64_t *lpx, const float *L, const int *flagoff,
                                                     float *tinv) {
  __shared__ float T11[TB * TB];
  __shared__ float Ti[TI];
  const int s = items[blockIdx.x].x, q = items[blockIdx.x].y;
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  const int nbd = (w + TB - 1) / TB, j = nbd - 1 - q;
  const int b0 = j * TB, m = min(TB, w - b0);
  const float *S = L + lpx[s];
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int cc = e / TB, r = e % TB;
    T11[r + cc * TB] = (r < m && cc < m) ? S[b0 + r + (size_t)(b0 + cc) * nrow] : 0.f;
  }
  __syncthreads();
  const int c = threadIdx.x;
  float x[TB];
#pragma unroll
  for (int k = 0; k < TB; ++k) x[k] = k == c ? 1.f : 0.f;
#pragma unroll
  for (int i = 1; i < TB; ++i) {
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) acc = fmaf(T11[i + k * TB], x[k], acc);
    if (i > c) x[i] = -acc;
  }
  float *base = tinv + (size_t)(flagoff[s] + j) * 3 * TI;
  float *out = base + (size_t)c * (TB + 1);
#pragma unroll
  for (int k = 0; k < TB; ++k) {
    const float v = (c < m && k < m) ? x[k] : 0.f;
    out[k] = v;
    Ti[c * (TB + 1) + k] = v;
  }
  out[TB] = 0.f;
  __syncthreads();
  // Mf(:, c) = T L(q, q-1)(:, c): the previous block is full (64 columns)
  {
    float g[TB];
#pragma unroll
    for (int k = 0; k < TB; ++k) g[k] = (j > 0 && k < m) ? S[b0 + k + (size_t)(b0 - TB + c) * nrow] : 0.f;
    float *o = base + TI + (size_t)c * (TB + 1);
#pragma unroll 4
    for (int rr = 0; rr < TB; ++rr) {
      float a = 0.f;
#pragma unroll
      for (int k = 0; k < TB; ++k) a = fmaf(Ti[k * (TB + 1) + rr], g[k], a);
      o[rr] = a;
    }
    o[TB] = 0.f;
  }
  // Mb(:, c) = T^T L(j+1, j)(c, :)^T: row c of the next block's tile
  {
    const int mn = j + 1 < nbd ? min(TB, w - b0 - TB) : 0;
    float h[TB];
#pragma unroll
    for (int k = 0; k < TB; ++k) h[k] = (c < mn && k < m) ? S[b0 + TB + c + (size_t)(b0 + k) * nrow] : 0.f;
    float *o = base + 2 * TI + (size_t)c * (TB + 1);
#pragma unroll 4
    for (int rr = 0; rr < TB; ++rr) {
      float a = 0.f;
#pragma unroll
      for (int k = 0; k < TB; ++k) a = fmaf(Ti[rr * (TB + 1) + k], h[k], a);
      o[rr] = a;
    }
    o[TB] = 0.f;
  }
}

// Matrix `part` (0: T, 1: Mf, 2: Mb) of diagonal tile (s, j) into shared
// memory (FP32 sweeps).
__device__ __forceinline__ void stage_inverse(const float *tinv, const int *flagoff, int s, int j, float *Ti,
                                              int part = 0) {
  const float4 *src = reinterpret_cast<const float4 *>(tinv + ((size_t)(flagoff[s] + j) * 3 + part) * TI);
  for (int e = threadIdx.x; e < TI / 4; e += blockDim.x) reinterpret_cast<float4 *>(Ti)[e] = __ldcg(src + e);
}

// Entries (r, c0 .. c0 + CPT - 1) of matrix `part` of diagonal tile (s, j),
// loaded at the start of an item so that the last link finds them in
// registers.
__device__ __forceinline__ void load_link(const float *tinv, const int *flagoff, int s, int j, int part, int r,
                                          int c0, float (&mv)[CPT]) {
  const float *src = tinv + ((size_t)(flagoff[s] + j) * 3 + part) * TI + (size_t)c0 * (TB + 1) + r;
#pragma unroll
  for (int cc = 0; cc < CPT; ++cc) mv[cc] = __ldcg(src + (size_t)cc * (TB + 1));
}

// The m x m tile at (b0, b0) of the panel, column-major in T11.
template <class T, class V> __device__ void stage_tile(const T *S, int nrow, int b0, int m, V *T11) {
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int c = e / TB, r = e % TB;
    T11[r + c * TB] = (r < m && c < m) ? V(S[b0 + r + (size_t)(b0 + c) * nrow]) : V(0);
  }
}

// Warp 0 only (all 32 lanes).  Forward flags of one supernode become ready
// in increasing block order; `front` = count of leading ready blocks.  Waits
// until block j is ready, scanning 32 flags per poll, and extends the front
// over ready blocks (< lim).  Waiters further from the front poll less often.
// Returns -1 on abort or timeout.
// With xws (the x words of the supernode's w columns; FP32 sweeps) the flag
// of block k is the epoch of the block's last word instead of fl[k], and no
// fence follows: the consumer reads the values as words and checks them.
__device__ int wait_up(const unsigned *fl, unsigned epoch, int j, int lim, int front, WideCtl *ctl, int *status,
                       const unsigned long long *xws = nullptr, int w = 0) {
  const int lane = threadIdx.x & 31;
  long long it = 0;
  const long long lim_ = wait_limit(ctl);
  volatile int *vab = &ctl->abort;
  while (true) {
    const int k = front + lane;
    unsigned v = 0u;
    if (k < lim)
      v = xws ? (unsigned)(*(volatile const unsigned long long *)(xws + min(w, (k + 1) * TB) - 1) >> 32)
              : *(volatile const unsigned *)(fl + k);
    const unsigned ready = __ballot_sync(0xffffffffu, v == epoch);
    const int lead = ready == 0xffffffffu ? 32 : __ffs(~ready) - 1;
    front += lead;
    if (lead == 32 && front < lim) continue;  // more ready flags to scan
    if (front > j) break;
    if (*vab) return -1;
    if (++it > lim_) {
      if (lane == 0) {
        atomicOr(status, ST_TIMEOUT);
        atomicExch(&ctl->abort, 1);
      }
      return -1;
    }
    __nanosleep(min(2000, 40 * (j - front + 1)));
  }
  if (!xws) __threadfence();
  return front;
}

// Backward mirror: blocks >= `front` are ready; waits until block i is and
// extends the front down to lo.
__device__ int wait_down(const unsigned *fl, unsigned epoch, int i, int lo, int front, WideCtl *ctl, int *status,
                         const unsigned long long *xws = nullptr, int w = 0) {
  const int lane = threadIdx.x & 31;
  long long it = 0;
  const long long lim_ = wait_limit(ctl);
  volatile int *vab = &ctl->abort;
  while (true) {
    const int k = front - 1 - lane;
    unsigned v = 0u;
    if (k >= lo)
      v = xws ? (unsigned)(*(volatile const unsigned long long *)(xws + min(w, (k + 1) * TB) - 1) >> 32)
              : *(volatile const unsigned *)(fl + k);
    const unsigned ready = __ballot_sync(0xffffffffu, v == epoch);
    const int lead = ready == 0xffffffffu ? 32 : __ffs(~ready) - 1;
    front -= lead;
    if (lead == 32 && front > lo) continue;
    if (front <= i) break;
    if (*vab) return -1;
    if (++it > lim_) {
      if (lane == 0) {
        atomicOr(status, ST_TIMEOUT);
        atomicExch(&ctl->abort, 1);
      }
      return -1;
    }
    __nanosleep(min(2000, 40 * (front - i)));
  }
  if (!xws) __threadfence();
  return front;
}

__device__ __forceinline__ void publish(unsigned *flag, unsigned epoch) {
  __threadfence();
  *(volatile unsigned *)flag = epoch;
}

// FP32 sweeps publish each solved x value as one 64-bit word (epoch << 32 |
// value bits): a consumer sees value and readiness in the same load, so
// neither side needs a fence or a flag.  Reads the n (<= CPT) words at wp
// into xv (0 beyond n), the whole warp polling until all of its lanes'
// words carry this epoch; false on abort or timeout.
template <int N>
__device__ __forceinline__ bool wait_words(const unsigned long long *wp, int n, unsigned epoch, float (&xv)[N],
                                           WideCtl *ctl, int *status) {
  long long it = 0;
  const long long lim_ = wait_limit(ctl);
  while (true) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      xv[k] = 0.f;
      if (k < n) {
        const unsigned long long v = *(volatile const unsigned long long *)(wp + k);
        if ((unsigned)(v >> 32) != epoch) ok = false;
        xv[k] = __uint_as_float((unsigned)v);
      }
    }
    if (__all_sync(0xffffffffu, ok)) return true;
    if (*(volatile int *)&ctl->abort) return false;
    if (++it > lim_) {
      if ((threadIdx.x & 31) == 0) {
        atomicOr(status, ST_TIMEOUT);
        atomicExch(&ctl->abort, 1);
      }
      return false;
    }
    __nanosleep(64);
  }
}
__device__ __forceinline__ void put_word(unsigned long long *wp, unsigned epoch, float v) {
  *(volatile unsigned long long *)wp = ((unsigned long long)epoch << 32) | __float_as_uint(v);
}

// Forward sweep over the large supernodes of one level.  Item (s, q): q <
// nbd(s) is diagonal block row q, else block q - nbd(s) of the rows below.
template <class T, class V>
__global__ void __launch_bounds__(SW_THREADS) k_fwd_blk(const int2 *items, int nitems, const int *super,
                                                        const int64_t *lpi, const int64_t *lpx, const int *ls,
                                                        const T *L, V *x, unsigned *flags, const int *flagoff,
                                                        unsigned epoch, const uint8_t *visible, WideCtl *ctl,
                                                        int *status, unsigned long long *xw, const float *tinv) {
  constexpr bool WORDS = sizeof(V) == 4;  // x of the diagonal blocks through words
  __shared__ __align__(16) V Td[TB * (TB + 1)];  // diagonal tile (FP32: its inverse)
  __shared__ V red[SW_THREADS];
  __shared__ V yb[TB];
  __shared__ int s_front;
  const int t = threadIdx.x, r = t & (TB - 1), cg = t / TB;
  int cur_s = -1, front = 0;
  bool failed = false;  // FP32 words: this thread saw a wait give up
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int s = items[it].x, q = items[it].y;
    if (visible && !visible[s]) continue;
    const int c0 = super[s], w = super[s + 1] - c0;
    const int nrow = (int)(lpi[s + 1] - lpi[s]);
    const T *S = L + lpx[s];
    unsigned *fl = flags + flagoff[s];
    V *xs = x + c0;
    if (s != cur_s) {
      cur_s = s;
      front = 0;
    }
    const int nbd = (w + TB - 1) / TB;
    const bool diag = q < nbd;
    const int r0 = diag ? q * TB : w + (q - nbd) * TB;
    const int m = min(TB, (diag ? w : nrow) - r0);
    // FP32 diagonal items leave block q - 1 to the last-link product
    const int jmax = diag ? (WORDS ? max(q - 1, 0) : q) : nbd;
    float mlink[CPT];  // FP32 diagonal items: this thread's entries of Mf_q
    if constexpr (WORDS) {
      if (diag) stage_inverse(tinv, flagoff, s, q, Td);
      if (diag && q > 0) load_link(tinv, flagoff, s, q, 1, r, cg * CPT, mlink);
    } else {
      if (diag) stage_tile(S, nrow, r0, m, Td);
    }
    // right-hand side of the block, final before this launch
    const V bq = (diag && t < m) ? __ldcg(xs + r0 + t) : V(0);
    const bool rok = r < m;
    const T *Lr = S + r0 + r;
    V acc = V(0);
    T v[CPT], vn[CPT];
#pragma unroll
    for (int cc = 0; cc < CPT; ++cc) {
      const int col = cg * CPT + cc;
      v[cc] = (jmax > 0 && rok && col < w) ? Lr[(size_t)col * nrow] : T(0);
    }
    for (int j = 0; j < jmax; ++j) {
      const int cbn = (j + 1) * TB + cg * CPT;
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc)
        vn[cc] = (j + 1 < jmax && rok && cbn + cc < w) ? Lr[(size_t)(cbn + cc) * nrow] : T(0);
      const int cb = j * TB + cg * CPT;
      if constexpr (WORDS) {
        if (j >= front) {
          __syncthreads();
          if (t < 32) {
            const int f = wait_up(fl, epoch, j, nbd, front, ctl, status, xw + c0, w);
            if (t == 0) s_front = f;
          }
          __syncthreads();
          front = s_front;
          if (front < 0) return;
        }
        float xv[CPT];
        if (!wait_words(xw + c0 + cb, min(CPT, w - cb), epoch, xv, ctl, status)) failed = true;
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc) acc += V(v[cc]) * xv[cc];
      } else {
        if (j >= front) {
          __syncthreads();
          if (t < 32) {
            const int f = wait_up(fl, epoch, j, nbd, front, ctl, status);
            if (t == 0) s_front = f;
          }
          __syncthreads();
          front = s_front;
          if (front < 0) return;
        }
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc)
          if (cb + cc < w) acc += V(v[cc]) * __ldcg(xs + cb + cc);
      }
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) v[cc] = vn[cc];
    }
    red[t] = acc;
    __syncthreads();
    if (t < TB) yb[t] = red[t] + red[t + TB] + red[t + 2 * TB] + red[t + 3 * TB];
    __syncthreads();
    if (diag) {
      if (t < m) yb[t] = bq - yb[t];
      __syncthreads();
      if constexpr (WORDS) {
        // c_q = T_q y_q (thread t < TB keeps entry t)
        V a = V(0);
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc)
          if (cg * CPT + cc < m) a += Td[(cg * CPT + cc) * (TB + 1) + r] * yb[cg * CPT + cc];
        red[t] = a;
        __syncthreads();
        const V cq = t < TB ? red[t] + red[t + TB] + red[t + 2 * TB] + red[t + 3 * TB] : V(0);
        __syncthreads();
        V xq = cq;
        if (q > 0) {
          // last link: x_q = c_q - Mf_q x_{q-1}, the words of block q - 1
          // polled directly by every warp
          const int cb = (q - 1) * TB + cg * CPT;
          float xv[CPT];
          if (!wait_words(xw + c0 + cb, CPT, epoch, xv, ctl, status)) failed = true;
          a = V(0);
#pragma unroll
          for (int cc = 0; cc < CPT; ++cc) a += mlink[cc] * xv[cc];
          red[t] = a;
          __syncthreads();
          if (t < TB) xq = cq - (red[t] + red[t + TB] + red[t + 2 * TB] + red[t + 3 * TB]);
        }
        if (t < m) {
          xs[r0 + t] = xq;
          put_word(xw + c0 + r0 + t, epoch, float(xq));
        }
      } else {
        if (t < 32) warp_trsv_lower(Td, m, yb);
        __syncthreads();
        if (t < m) xs[r0 + t] = yb[t];
        __syncthreads();
        if (t == 0) publish(fl + q, epoch);
      }
    } else {
      const int *rows = ls + lpi[s];
      if (t < m) atomicAdd(&x[rows[r0 + t]], -yb[t]);
    }
    if (__syncthreads_or(failed)) return;  // a wait gave up (all warps leave together)
  }
}

// Backward sweep over the large supernodes of one level.  Item (s, q) is
// column block j = nbd(s) - 1 - q.
template <class T, class V>
__global__ void __launch_bounds__(SW_THREADS) k_bwd_blk(const int2 *items, int nitems, const int *super,
                                                        const int64_t *lpi, const int64_t *lpx, const int *ls,
                                                        const T *L, V *x, unsigned *flags, const int *flagoff,
                                                        unsigned epoch, const uint8_t *visible, WideCtl *ctl,
                                                        int *status, unsigned long long *xw, const float *tinv) {
  constexpr bool WORDS = sizeof(V) == 4;  // x of the diagonal blocks through words
  __shared__ __align__(16) V Td[TB * (TB + 1)];  // diagonal tile (FP32: its inverse)
  __shared__ V red[2][TB];
  __shared__ V redS[sizeof(V) == 4 ? TB * (TB + 1) : 1];  // FP32: column sums through a transpose
  __shared__ V yb[TB];
  __shared__ int s_front;
  const int t = threadIdx.x, r = t & (TB - 1), cg = t / TB, lane = t & 31;
  int cur_s = -1, front = 0;
  bool failed = false;  // FP32 words: this thread saw a wait give up
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int s = items[it].x, q = items[it].y;
    if (visible && !visible[s]) continue;
    const int c0 = super[s], w = super[s + 1] - c0;
    const int nrow = (int)(lpi[s + 1] - lpi[s]);
    const T *S = L + lpx[s];
    const int *rows = ls + lpi[s];
    unsigned *fl = flags + flagoff[s];
    V *xs = x + c0;
    const int nbd = (w + TB - 1) / TB;
    if (s != cur_s) {
      cur_s = s;
      front = nbd;
    }
    const int j = nbd - 1 - q;
    const int b0 = j * TB, nc = min(TB, w - b0);
    float mlink[CPT];  // FP32: this thread's entries of Mb_j
    if constexpr (WORDS) {
      stage_inverse(tinv, flagoff, s, j, Td);
      if (j + 1 < nbd) load_link(tinv, flagoff, s, j, 2, r, cg * CPT, mlink);
    } else {
      stage_tile(S, nrow, b0, nc, Td);
    }
    const int cb = b0 + cg * CPT;
    const T *Lc = S + (size_t)cb * nrow;  // first of this thread's columns
    bool cok[CPT];
#pragma unroll
    for (int cc = 0; cc < CPT; ++cc) cok[cc] = cb + cc < w;
    V part[CPT];
#pragma unroll
    for (int cc = 0; cc < CPT; ++cc) part[cc] = V(0);
    // rows below the diagonal block: x known from the ancestors; four rows
    // per step so that their index and value loads are in flight together
    int row = w + r;
    for (; row + 3 * TB < nrow; row += 4 * TB) {
      const int i0 = rows[row], i1 = rows[row + TB], i2 = rows[row + 2 * TB], i3 = rows[row + 3 * TB];
      const V x0 = __ldcg(x + i0), x1 = __ldcg(x + i1), x2 = __ldcg(x + i2), x3 = __ldcg(x + i3);
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc)
        if (cok[cc]) {
          const T *lp = Lc + row + (size_t)cc * nrow;
          part[cc] += V(lp[0]) * x0;
          part[cc] += V(lp[TB]) * x1;
          part[cc] += V(lp[2 * TB]) * x2;
          part[cc] += V(lp[3 * TB]) * x3;
        }
    }
    for (; row < nrow; row += TB) {
      const V xv = __ldcg(x + rows[row]);
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc)
        if (cok[cc]) part[cc] += V(Lc[row + (size_t)cc * nrow]) * xv;
    }
    // diagonal-block rows of later blocks, in the order they become ready
    // (FP32: block j + 1 is left to the last-link product)
    const int ilo = WORDS ? j + 1 : j;  // blocks i > ilo
    T v[CPT], vn[CPT];
    {
      const int row = (nbd - 1) * TB + r;
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) v[cc] = (ilo < nbd - 1 && row < w && cok[cc]) ? Lc[row + (size_t)cc * nrow] : T(0);
    }
    for (int i = nbd - 1; i > ilo; --i) {
      const int rown = (i - 1) * TB + r;
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc)
        vn[cc] = (i - 1 > ilo && rown < w && cok[cc]) ? Lc[rown + (size_t)cc * nrow] : T(0);
      const int row = i * TB + r;
      V xv;
      if constexpr (WORDS) {
        if (i < front) {
          __syncthreads();
          if (t < 32) {
            const int f = wait_down(fl, epoch, i, j + 1, front, ctl, status, xw + c0, w);
            if (t == 0) s_front = f;
          }
          __syncthreads();
          front = s_front;
          if (front < 0) return;
        }
        float xw1[1];
        if (!wait_words(xw + c0 + row, row < w ? 1 : 0, epoch, xw1, ctl, status)) failed = true;
        xv = xw1[0];
      } else {
        if (i < front) {
          __syncthreads();
          if (t < 32) {
            const int f = wait_down(fl, epoch, i, j + 1, front, ctl, status);
            if (t == 0) s_front = f;
          }
          __syncthreads();
          front = s_front;
          if (front < 0) return;
        }
        xv = row < w ? __ldcg(xs + row) : V(0);
      }
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) part[cc] += V(v[cc]) * xv;
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) v[cc] = vn[cc];
    }
    // column sums over the 64 rows
    if constexpr (sizeof(V) == 4) {
      // transpose through shared memory, then one thread per column
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) redS[(cg * CPT + cc) * (TB + 1) + r] = part[cc];
      __syncthreads();
      if (t < nc) {
        const V *col = redS + t * (TB + 1);
        V a0 = V(0), a1 = V(0), a2 = V(0), a3 = V(0);
#pragma unroll
        for (int k = 0; k < TB; k += 4) {
          a0 += col[k];
          a1 += col[k + 1];
          a2 += col[k + 2];
          a3 += col[k + 3];
        }
        yb[t] = __ldcg(xs + b0 + t) - ((a0 + a1) + (a2 + a3));
      }
    } else {
      // warps 2cg and 2cg+1 hold rows 0-31, 32-63
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc) {
        V a = part[cc];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[(t >> 5) & 1][cg * CPT + cc] = a;
      }
      __syncthreads();
      if (t < nc) yb[t] = __ldcg(xs + b0 + t) - (red[0][t] + red[1][t]);
    }
    __syncthreads();
    if constexpr (WORDS) {
      // c_j = T_j^T y_j (thread t < TB keeps entry t)
      V a = V(0);
#pragma unroll
      for (int cc = 0; cc < CPT; ++cc)
        if (cg * CPT + cc < nc) a += Td[r * (TB + 1) + cg * CPT + cc] * yb[cg * CPT + cc];
      redS[t] = a;
      __syncthreads();
      const V cj = t < TB ? redS[t] + redS[t + TB] + redS[t + 2 * TB] + redS[t + 3 * TB] : V(0);
      __syncthreads();
      V xj = cj;
      if (j + 1 < nbd) {
        // last link: x_j = c_j - Mb_j x_{j+1}, the words of block j + 1
        // polled directly by every warp
        const int cb1 = (j + 1) * TB + cg * CPT;
        float xv[CPT];
        if (!wait_words(xw + c0 + cb1, min(CPT, w - cb1), epoch, xv, ctl, status)) failed = true;
        a = V(0);
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc) a += mlink[cc] * xv[cc];
        redS[t] = a;
        __syncthreads();
        if (t < TB) xj = cj - (redS[t] + redS[t + TB] + redS[t + 2 * TB] + redS[t + 3 * TB]);
      }
      if (t < nc) {
        xs[b0 + t] = xj;
        put_word(xw + c0 + b0 + t, epoch, float(xj));
      }
    } else {
      if (t < 32) warp_trsv_lower_t(Td, nc, yb);
      __syncthreads();
      if (t < nc) xs[b0 + t] = yb[t];
      __syncthreads();
      if (t == 0) publish(fl + j, epoch);
    }
    if (__syncthreads_or(failed)) return;  // a wait gave up (all warps leave together)
  }
}

template <class K> static int coop_grid(Plan &P, K kern, int items) {
  int occ = 0;
  NQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, SW_THREADS, 0));
  occ = std::max(occ, 1);
  return std::max(1, std::min(items, occ * std::max(1, P.num_sms)));
}

// Next launch epoch of the ready flags (0 never marks a ready block).
static unsigned next_epoch(Plan &P) {
  if (++P.solve_epoch == 0) {
    cudaMemsetAsync(P.d_solve_flags, 0, P.solve_flags_cap * sizeof(unsigned), P.stream);
    cudaMemsetAsync(P.d_xw, 0, (size_t)std::max(P.n, 1) * sizeof(unsigned long long), P.stream);
    P.solve_epoch = 1;
  }
  return P.solve_epoch;
}

}  // namespace

template <class T, class V> static int launch_blk(Plan &P, bool fwd, int l, const T *L, V *x) {
  const int off = fwd ? P.blk_fwd_off[l] : P.blk_bwd_off[l];
  const int cnt = (fwd ? P.blk_fwd_off[l + 1] : P.blk_bwd_off[l + 1]) - off;
  if (cnt <= 0) return NQG_OK;
  const int2 *items = reinterpret_cast<const int2 *>(P.d_blk_items) + off;
  WideCtl *ctl = reinterpret_cast<WideCtl *>(P.d_wide_ctl);
  int *status = P.d_status;
  unsigned *flags = P.d_solve_flags;
  const int *flagoff = P.d_flagoff;
  const uint8_t *vis = P.masked ? P.d_visible : nullptr;
  const int *super = P.d_super, *ls = P.d_ls;
  const int64_t *lpi = P.d_lpi, *lpx = P.d_lpx;
  NQG_CUDA(cudaMemsetAsync(ctl, 0, 16, P.stream));
  unsigned epoch = next_epoch(P);
  void *kern = fwd ? (void *)k_fwd_blk<T, V> : (void *)k_bwd_blk<T, V>;
  const int G = fwd ? coop_grid(P, k_fwd_blk<T, V>, cnt) : coop_grid(P, k_bwd_blk<T, V>, cnt);
  unsigned long long *xw = P.d_xw;
  const float *tinv = reinterpret_cast<const float *>(P.d_tinv);
  if constexpr (sizeof(V) == 4) {
    if (!tinv) return NQG_ERR_ARG;
    // inverses of the diagonal tiles, once per factorization
    if (!P.tinv_valid) {
      const int nb_all = P.blk_bwd_off.back() - P.blk_bwd_off.front();
      if (nb_all > 0) {
        cudaEvent_t ei = P.prof_begin();
        k_tile_inverse<<<nb_all, TB, 0, P.stream>>>(reinterpret_cast<const int2 *>(P.d_blk_items) +
                                                        P.blk_bwd_off.front(),
                                                    super, lpi, lpx, reinterpret_cast<const float *>(L), flagoff,
                                                    P.d_tinv);
        NQG_CUDA(cudaGetLastError());
        P.nlaunch++;
        P.prof_end(NQG_K_SOLVE, ei, 0.0, 0.0);
      }
      P.tinv_valid = true;
    }
  }
  void *args[] = {(void *)&items, (void *)&cnt, (void *)&super, (void *)&lpi, (void *)&lpx, (void *)&ls,
                  (void *)&L, &x, &flags, (void *)&flagoff, &epoch, (void *)&vis, &ctl, &status, &xw, &tinv};
  cudaEvent_t e0 = P.prof_begin();
  NQG_CUDA(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(SW_THREADS), args, 0, P.stream));
  P.nlaunch++;
  P.prof_end(NQG_K_SOLVE, e0, 0.0, P.prof ? P.blk_bytes[l] * (double)sizeof(T) : 0.0);
  return NQG_OK;
}

template <class T, class V> int solve_blk_fwd(Plan &P, int l, const T *L, V *x) {
  return launch_blk<T, V>(P, true, l, L, x);
}
template <class T, class V> int solve_blk_bwd(Plan &P, int l, const T *L, V *x) {
  return launch_blk<T, V>(P, false, l, L, x);
}

template int solve_blk_fwd<float, float>(Plan &, int, const float *, float *);
template int solve_blk_fwd<float, double>(Plan &, int, const float *, double *);
template int solve_blk_fwd<double, double>(Plan &, int, const double *, double *);
template int solve_blk_bwd<float, float>(Plan &, int, const float *, float *);
template int solve_blk_bwd<float, double>(Plan &, int, const float *, double *);
template int solve_blk_bwd<double, double>(Plan &, int, const double *, double *);

}  // namespace nqg
