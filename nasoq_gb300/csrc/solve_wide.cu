// Forward and backward supernodal solves for one wide supernode, spread over
// the whole GPU (reference H2LeveledBlockedLsolve / LTsolve per supernode,
// src/triangularSolve/Triangular_BCSC.cpp:378-446, 534-600: dtrsm on the
// diagonal block + dgemv with the rows below).
//
// The w x w unit-lower diagonal block is processed in 64-column blocks with
// one grid barrier per block: after x_b is known, CTA 0 applies it to the next
// block's 64 rows (look-ahead) and solves that block's triangle in a single
// warp from shared memory, while the other CTAs apply x_b to all later rows.
// The rows below the diagonal block form one independent GEMV (forward) or
// GEMV^T (backward) over (row, column-chunk) items.  Each row (forward) or
// column (backward) of the block keeps one owner thread in every phase.
#include <cuda_runtime.h>

#include <algorithm>

#include "coop.cuh"
#include "plan.hpp"

namespace nqg {

namespace {

constexpr int SW_THREADS = 256;
constexpr int SB = 64;      // diagonal sub-block size
constexpr int CHUNK = 512;  // column chunk of the below-block GEMV

// x_b := L11[b]^-1 x_b for a 64x64 unit lower block, one warp, lane i holds
// rows i and i+32; T11 is the block staged column-major in shared memory.
__device__ void warp_trsv_lower(const double *T11, int m, double *xb) {
  const int lane = threadIdx.x & 31;
  double v0 = lane < m ? xb[lane] : 0.0, v1 = lane + 32 < m ? xb[lane + 32] : 0.0;
  for (int j = 0; j < m; ++j) {
    const double xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31);
    if (lane > j && lane < m) v0 -= T11[lane + j * SB] * xj;
    if (lane + 32 > j && lane + 32 < m) v1 -= T11[lane + 32 + j * SB] * xj;
  }
  if (lane < m) xb[lane] = v0;
  if (lane + 32 < m) xb[lane + 32] = v1;
}

// x_b := L11[b]^-T x_b (backward substitution with the transposed block).
__device__ void warp_trsv_lower_t(const double *T11, int m, double *xb) {
  const int lane = threadIdx.x & 31;
  double v0 = lane < m ? xb[lane] : 0.0, v1 = lane + 32 < m ? xb[lane + 32] : 0.0;
  for (int i = m - 1; i > 0; --i) {
    const double xi = __shfl_sync(0xffffffffu, i < 32 ? v0 : v1, i & 31);
    // x_j -= L(i, j) x_i for j < i
    if (lane < i) v0 -= T11[i + lane * SB] * xi;
    if (lane + 32 < i) v1 -= T11[i + (lane + 32) * SB] * xi;
  }
  if (lane < m) xb[lane] = v0;
  if (lane + 32 < m) xb[lane + 32] = v1;
}

template <class T> __device__ void stage_block(const T *S, int nrow, int b0, int m, double *T11) {
  for (int e = threadIdx.x; e < SB * SB; e += blockDim.x) {
    int c = e / SB, r = e % SB;
    T11[r + c * SB] = (r < m && c < m) ? (double)S[b0 + r + (size_t)(b0 + c) * nrow] : 0.0;
  }
}

template <class T>
__global__ void __launch_bounds__(SW_THREADS) k_fwd_wide(const T *S, int nrow, int w, const int *rows, double *x,
                                                         int c0, WideCtl *ctl, int *status) {
  __shared__ double T11[SB * SB];
  __shared__ double xb[SB], xn[SB];
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, TT = gridDim.x * blockDim.x;
  const int nblk = (w + SB - 1) / SB;
  double *xs = x + c0;
  auto first_row = [&](int lo) { return lo + (int)(((long long)gt - lo % TT + TT) % TT); };
  if (blockIdx.x == 0) {  // first diagonal block
    const int m = min(SB, w);
    stage_block(S, nrow, 0, m, T11);
    for (int i = threadIdx.x; i < m; i += blockDim.x) xb[i] = xs[i];
    __syncthreads();
    if (threadIdx.x < 32) warp_trsv_lower(T11, m, xb);
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) xs[i] = xb[i];
  }
  if (!grid_sync(ctl, status)) return;
  for (int b = 0; b < nblk; ++b) {
    const int b0 = b * SB, b1 = min(w, b0 + SB), b2 = min(w, b1 + SB);
    const int m = b1 - b0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) xb[i] = xs[b0 + i];
    __syncthreads();
    if (blockIdx.x == 0 && b1 < w) {
      // look-ahead: rows [b1, b2) get block b, then their triangle is solved
      for (int r = b1 + threadIdx.x; r < b2; r += blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < m; ++j) acc += (double)S[r + (size_t)(b0 + j) * nrow] * xb[j];
        xs[r] -= acc;
      }
      __syncthreads();
      const int m2 = b2 - b1;
      stage_block(S, nrow, b1, m2, T11);
      for (int i = threadIdx.x; i < m2; i += blockDim.x) xn[i] = xs[b1 + i];
      __syncthreads();
      if (threadIdx.x < 32) warp_trsv_lower(T11, m2, xn);
      __syncthreads();
      for (int i = threadIdx.x; i < m2; i += blockDim.x) xs[b1 + i] = xn[i];
    }
    // every CTA (CTA 0 included) applies block b to its rows beyond the look-ahead
    for (int r = first_row(b2); r < w; r += TT) {
      double acc = 0.0;
      for (int j = 0; j < m; ++j) acc += (double)S[r + (size_t)(b0 + j) * nrow] * xb[j];
      xs[r] -= acc;
    }
    if (!grid_sync(ctl, status)) return;
  }
  // rows below the diagonal block: x[rows[r]] -= L21(r, :) x_s, split in column chunks
  const int nb_rows = nrow - w;
  const int nchunk = (w + CHUNK - 1) / CHUNK;
  for (long long item = gt; item < (long long)nb_rows * nchunk; item += TT) {
    const int r = w + (int)(item % nb_rows);
    const int ch = (int)(item / nb_rows);
    const int j0 = ch * CHUNK, j1 = min(w, j0 + CHUNK);
    double acc = 0.0;
    for (int j = j0; j < j1; ++j) acc += (double)S[r + (size_t)j * nrow] * xs[j];
    atomicAdd(&x[rows[r]], -acc);
  }
}

template <class T>
__global__ void __launch_bounds__(SW_THREADS) k_bwd_wide(const T *S, int nrow, int w, const int *rows, double *x,
                                                         int c0, WideCtl *ctl, int *status) {
  __shared__ double T11[SB * SB];
  __shared__ double xb[SB], xn[SB];
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, TT = gridDim.x * blockDim.x;
  const int nblk = (w + SB - 1) / SB;
  double *xs = x + c0;
  auto first_col = [&](int lo) { return lo + (int)(((long long)gt - lo % TT + TT) % TT); };
  // x_s -= L21^T x(rows below), (column, row-chunk) items
  const int nb_rows = nrow - w;
  if (nb_rows > 0) {
    const int nchunk = (nb_rows + CHUNK - 1) / CHUNK;
    for (long long item = gt; item < (long long)w * nchunk; item += TT) {
      const int j = (int)(item % w);
      const int ch = (int)(item / w);
      const int r0 = w + ch * CHUNK, r1 = min(nrow, r0 + CHUNK);
      double acc = 0.0;
      for (int r = r0; r < r1; ++r) acc += (double)S[r + (size_t)j * nrow] * x[rows[r]];
      atomicAdd(&xs[j], -acc);
    }
  }
  if (!grid_sync(ctl, status)) return;
  // last diagonal block
  const int lb0 = (nblk - 1) * SB;
  if (blockIdx.x == 0) {
    const int m = w - lb0;
    stage_block(S, nrow, lb0, m, T11);
    for (int i = threadIdx.x; i < m; i += blockDim.x) xb[i] = xs[lb0 + i];
    __syncthreads();
    if (threadIdx.x < 32) warp_trsv_lower_t(T11, m, xb);
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) xs[lb0 + i] = xb[i];
  }
  if (!grid_sync(ctl, status)) return;
  for (int b = nblk - 1; b > 0; --b) {
    const int b0 = b * SB, b1 = min(w, b0 + SB);
    const int m = b1 - b0;
    const int p0 = b0 - SB;  // previous block [p0, b0)
    for (int i = threadIdx.x; i < m; i += blockDim.x) xb[i] = xs[b0 + i];
    __syncthreads();
    if (blockIdx.x == 0) {
      // look-ahead: columns [p0, b0) get block b, then their triangle is solved
      for (int j = p0 + threadIdx.x; j < b0; j += blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < m; ++i) acc += (double)S[b0 + i + (size_t)j * nrow] * xb[i];
        xs[j] -= acc;
      }
      __syncthreads();
      stage_block(S, nrow, p0, SB, T11);
      for (int i = threadIdx.x; i < SB; i += blockDim.x) xn[i] = xs[p0 + i];
      __syncthreads();
      if (threadIdx.x < 32) warp_trsv_lower_t(T11, SB, xn);
      __syncthreads();
      for (int i = threadIdx.x; i < SB; i += blockDim.x) xs[p0 + i] = xn[i];
    }
    // every CTA (CTA 0 included) applies block b to its columns before the look-ahead
    for (int j = first_col(0); j < p0; j += TT) {
      double acc = 0.0;
      for (int i = 0; i < m; ++i) acc += (double)S[b0 + i + (size_t)j * nrow] * xb[i];
      xs[j] -= acc;
    }
    if (!grid_sync(ctl, status)) return;
  }
}

}  // namespace

template <class T> int solve_wide_fwd(Plan &P, int s, const T *L, double *x) {
  const int c0 = P.sym.super[s], w = P.sym.super[s + 1] - c0;
  const int nrow = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
  const T *S = L + P.sym.lpx[s];
  const int *rows = P.d_ls + P.sym.lpi[s];
  WideCtl *ctl = reinterpret_cast<WideCtl *>(P.d_wide_ctl);
  int *status = P.d_status;
  NQG_CUDA(cudaMemsetAsync(ctl, 0, 16, P.stream));
  int G = std::max(1, P.num_sms);
  void *args[] = {(void *)&S, (void *)&nrow, (void *)&w, (void *)&rows, &x, (void *)&c0, &ctl, &status};
  cudaEvent_t e0 = P.prof_begin();
  NQG_CUDA(cudaLaunchCooperativeKernel((void *)k_fwd_wide<T>, dim3(G), dim3(SW_THREADS), args, 0, P.stream));
  P.nlaunch++;
  P.prof_end(NQG_K_SOLVE, e0, 0.0, (double)nrow * w * sizeof(T));
  return NQG_OK;
}

template <class T> int solve_wide_bwd(Plan &P, int s, const T *L, double *x) {
  const int c0 = P.sym.super[s], w = P.sym.super[s + 1] - c0;
  const int nrow = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
  const T *S = L + P.sym.lpx[s];
  const int *rows = P.d_ls + P.sym.lpi[s];
  WideCtl *ctl = reinterpret_cast<WideCtl *>(P.d_wide_ctl);
  int *status = P.d_status;
  NQG_CUDA(cudaMemsetAsync(ctl, 0, 16, P.stream));
  int G = std::max(1, P.num_sms);
  void *args[] = {(void *)&S, (void *)&nrow, (void *)&w, (void *)&rows, &x, (void *)&c0, &ctl, &status};
  cudaEvent_t e0 = P.prof_begin();
  NQG_CUDA(cudaLaunchCooperativeKernel((void *)k_bwd_wide<T>, dim3(G), dim3(SW_THREADS), args, 0, P.stream));
  P.nlaunch++;
  P.prof_end(NQG_K_SOLVE, e0, 0.0, (double)nrow * w * sizeof(T));
  return NQG_OK;
}

template int solve_wide_fwd<float>(Plan &, int, const float *, double *);
template int solve_wide_fwd<double>(Plan &, int, const double *, double *);
template int solve_wide_bwd<float>(Plan &, int, const float *, double *);
template int solve_wide_bwd<double>(Plan &, int, const double *, double *);

}  // namespace nqg
