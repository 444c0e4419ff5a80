// Supernodal forward / diagonal / backward solves, the symmetric SpMV of the
// refinement residual, and the FP64 restarted GMRES refinement loop.
//
// Forward (reference H2LeveledBlockedLsolve, src/triangularSolve/
// Triangular_BCSC.cpp:378-446): per level, one CTA per supernode solves its
// unit-lower diagonal block and scatters L21 x1 into the rows below with
// atomics.  Diagonal: 1x1 scaling by 1/d, 2x2 blocks by Cramer's rule
// (blocked_2by2_solver, src/common/Sym_BLAS.cpp:492-529).  Backward
// (H2LeveledBlockedLTsolve, Triangular_BCSC.cpp:534-600): per level in
// reverse, gather x(rows below), x1 -= L21^T x2, then the transposed unit
// triangle.  Vectors are FP64; factor values are FP64 or FP32 (FP32 values
// are widened before use).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "plan.hpp"

namespace nqg {

namespace {

constexpr int SV_THREADS = 256;

template <class T, class V>
__global__ void __launch_bounds__(SV_THREADS) k_fwd(const int *targets, const int *super, const int64_t *lpi,
                                                    const int64_t *lpx, const int *ls, const T *L, V *x,
                                                    const uint8_t *visible) {
  extern __shared__ __align__(16) unsigned char sv_raw[];
  V *xs = reinterpret_cast<V *>(sv_raw);
  const int s = targets[blockIdx.x];
  if (visible && !visible[s]) return;
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  const T *Ls = L + lpx[s];
  for (int i = threadIdx.x; i < w; i += blockDim.x) xs[i] = x[c0 + i];
  __syncthreads();
  for (int j = 0; j < w - 1; ++j) {
    const V xj = xs[j];
    for (int i = j + 1 + threadIdx.x; i < w; i += blockDim.x) xs[i] -= V(Ls[i + (size_t)j * nrow]) * xj;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < w; i += blockDim.x) x[c0 + i] = xs[i];
  const int *rows = ls + lpi[s];
  for (int r = w + threadIdx.x; r < nrow; r += blockDim.x) {
    V y = V(0);
    for (int j = 0; j < w; ++j) y += V(Ls[r + (size_t)j * nrow]) * xs[j];
    atomicAdd(&x[rows[r]], -y);
  }
}

template <class T, class V>
__global__ void k_dsolve(int n, const T *Dg, V *x, const uint8_t *hidden) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (hidden && hidden[i]) continue;
    const V e = V(Dg[n + i]);
    if (i > 0 && Dg[n + i - 1] != T(0) && !(hidden && hidden[i - 1])) continue;  // second of a 2x2 block
    if (e == V(0)) {
      x[i] *= V(1) / V(Dg[i]);
    } else {
      const V d1 = V(Dg[i]), d2 = V(Dg[i + 1]);
      const V inv = V(1) / (d1 * d2 - e * e);
      const V x1 = x[i], x2 = x[i + 1];
      x[i] = (x1 * d2 - x2 * e) * inv;
      x[i + 1] = (x2 * d1 - x1 * e) * inv;
    }
  }
}

template <class T, class V>
__global__ void __launch_bounds__(SV_THREADS) k_bwd(const int *targets, const int *super, const int64_t *lpi,
                                                    const int64_t *lpx, const int *ls, const T *L, V *x,
                                                    const uint8_t *visible) {
  extern __shared__ __align__(16) unsigned char sv_raw[];
  V *xs = reinterpret_cast<V *>(sv_raw);
  const int s = targets[blockIdx.x];
  if (visible && !visible[s]) return;
  const int c0 = super[s], w = super[s + 1] - c0;
  const int nrow = (int)(lpi[s + 1] - lpi[s]);
  const T *Ls = L + lpx[s];
  const int *rows = ls + lpi[s];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < w; i += blockDim.x) xs[i] = x[c0 + i];
  __syncthreads();
  // x1 -= L21^T x2: one warp per column
  for (int j = wid; j < w; j += nw) {
    V acc = V(0);
    for (int r = w + lane; r < nrow; r += 32) acc += V(Ls[r + (size_t)j * nrow]) * x[rows[r]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) xs[j] -= acc;
  }
  __syncthreads();
  // transposed unit triangle, column sweep from the last column
  for (int i = w - 1; i > 0; --i) {
    const V xi = xs[i];
    for (int j = threadIdx.x; j < i; j += blockDim.x) xs[j] -= V(Ls[i + (size_t)j * nrow]) * xi;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < w; i += blockDim.x) x[c0 + i] = xs[i];
}

// y_ord = (P K P^T) x_ord using the full CSR R of K in the original
// ordering: y_ord[i] = sum_k R(perm[i], j_k) x_ord[iperm[j_k]].
__global__ void k_spmv_ord(int n, const int *Rp, const int *Rj, const double *Rx, const int *perm, const int *iperm,
                           const double *xo, double *yo) {
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int row = perm[i];
    double acc = 0.0;
    for (int q = Rp[row] + lane; q < Rp[row + 1]; q += 32) acc += Rx[q] * xo[iperm[Rj[q]]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) yo[i] = acc;
  }
}

__global__ void k_spmv_orig(int n, const int *Rp, const int *Rj, const double *Rx, const double *x, double *y) {
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    double acc = 0.0;
    for (int q = Rp[i] + lane; q < Rp[i + 1]; q += 32) acc += Rx[q] * x[Rj[q]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[i] = acc;
  }
}

__global__ void k_narrow(int n, const double *src, float *dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (float)src[i];
}
__global__ void k_widen(int n, const float *src, double *dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (double)src[i];
}
__global__ void k_gather(int n, const int *perm, const double *src, double *dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[perm[i]];
}
__global__ void k_scatter(int n, const int *perm, const double *src, double *dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[perm[i]] = src[i];
}
__global__ void k_sub(int n, const double *a, double *b) {  // b = a - b
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i] - b[i];
}
__global__ void k_axpy(int n, const double *alpha_p, double sign, const double *x, double *y) {
  const double a = sign * *alpha_p;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += a * x[i];
}
__global__ void k_scale_div(int n, const double *den_p, const double *x, double *y) {
  const double d = *den_p;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = x[i] / d;
}
// x += V y  (k+1 basis vectors)
__global__ void k_update_x(int n, int kp1, const double *V, const double *y, double *x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = x[i];
    for (int j = 0; j < kp1; ++j) acc += V[(size_t)j * n + i] * y[j];
    x[i] = acc;
  }
}

// x += Z y with FP32 preconditioned directions Z (k+1 of them)
__global__ void k_update_x_f(int n, int kp1, const float *Z, const double *y, double *x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = x[i];
    for (int j = 0; j < kp1; ++j) acc += (double)Z[(size_t)j * n + i] * y[j];
    x[i] = acc;
  }
}

// Deterministic two-stage dot product: partial sums per block, then one block.
constexpr int DOT_BLOCKS = 256;
__global__ void k_dot_partial(int n, const double *a, const double *b, double *part) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += a[i] * b[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
  }
}
__global__ void k_dot_final(const double *part, int np, double *out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *out = acc;
  }
}

inline int grid_for(int n) { return std::max(1, std::min((n + 255) / 256, 2048)); }

}  // namespace

template <class T, class V> static int ldlt_solve_impl(Plan &P, V *x) {
  cudaStream_t st = P.stream;
  const T *L = reinterpret_cast<const T *>(P.d_L);
  const T *D = reinterpret_cast<const T *>(P.d_D);
  const uint8_t *vis = P.masked ? P.d_visible : nullptr;
  const uint8_t *hid = P.masked ? P.d_hidden : nullptr;
  // small supernodes only (the others take the block kernels)
  const size_t smem = (size_t)std::max(std::min(P.sym.max_sup_wid, P.solve_small_w), 1) * sizeof(V);
  if (smem > 227 * 1024) return NQG_ERR_SIZE;
  if (smem > 48 * 1024) {
    NQG_CUDA(cudaFuncSetAttribute(k_fwd<T, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    NQG_CUDA(cudaFuncSetAttribute(k_bwd<T, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int nlev = (int)P.levels.size();
  int rc;
  auto lvl_bytes = [&](int l) {
    double b = 0;
    if (P.prof)
      for (int q = P.level_off[l]; q < P.level_off[l + 1]; ++q) {
        int s = P.lv_targets_host[q];
        b += (double)(P.sym.lpi[s + 1] - P.sym.lpi[s]) * (P.sym.super[s + 1] - P.sym.super[s]) * sizeof(T);
      }
    return b;
  };
  for (int l = 0; l < nlev; ++l) {
    int cnt = P.level_off[l + 1] - P.level_off[l];
    if (cnt > 0) {
      cudaEvent_t e0 = P.prof_begin();
      k_fwd<T, V><<<cnt, SV_THREADS, smem, st>>>(P.d_targets_lv + P.level_off[l], P.d_super, P.d_lpi, P.d_lpx, P.d_ls,
                                               L, x, vis);
      P.prof_end(NQG_K_SOLVE, e0, 0.0, lvl_bytes(l));
      P.nlaunch++;
    }
    if ((rc = solve_blk_fwd<T, V>(P, l, L, x))) return rc;
  }
  k_dsolve<T, V><<<grid_for(P.n), 256, 0, st>>>(P.n, D, x, hid);
  P.nlaunch++;
  for (int l = nlev - 1; l >= 0; --l) {
    if ((rc = solve_blk_bwd<T, V>(P, l, L, x))) return rc;
    int cnt = P.level_off[l + 1] - P.level_off[l];
    if (cnt > 0) {
      cudaEvent_t e0 = P.prof_begin();
      k_bwd<T, V><<<cnt, SV_THREADS, smem, st>>>(P.d_targets_lv + P.level_off[l], P.d_super, P.d_lpi, P.d_lpx, P.d_ls,
                                               L, x, vis);
      P.prof_end(NQG_K_SOLVE, e0, 0.0, lvl_bytes(l));
      P.nlaunch++;
    }
  }
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

// FP32 factors: with solve_precision FP32 the triangular solves run in FP32
// (the vector is narrowed on the way in and widened on the way out), else the
// factor entries are widened and the solves run in FP64.  The refinement
// around them is FP64 either way.
int dev_ldlt_solve_ord(Plan &P, double *d_x) {
  if (P.set.precision == NQG_FP32) {
    if (P.set.solve_precision != NQG_FP32) return ldlt_solve_impl<float, double>(P, d_x);
    k_narrow<<<grid_for(P.n), 256, 0, P.stream>>>(P.n, d_x, P.d_xf);
    P.nlaunch++;
    int rc = ldlt_solve_impl<float, float>(P, P.d_xf);
    if (rc) return rc;
    k_widen<<<grid_for(P.n), 256, 0, P.stream>>>(P.n, P.d_xf, d_x);
    P.nlaunch++;
    return NQG_OK;
  }
  return ldlt_solve_impl<double, double>(P, d_x);
}

int dev_spmv_ord(Plan &P, const double *xo, double *yo) {
  int blocks = std::max(1, std::min((P.n + 7) / 8, 8192));
  cudaEvent_t e0 = P.prof_begin();
  k_spmv_ord<<<blocks, 256, 0, P.stream>>>(P.n, P.d_Rp, P.d_Rj, P.d_Rx, P.d_perm, P.d_iperm, xo, yo);
  // values + column indices, row pointers, x gathered through iperm, y, perm/iperm
  P.prof_end(NQG_K_SPMV, e0, 2.0 * P.nnzR, 12.0 * P.nnzR + 4.0 * (P.n + 1) + 24.0 * P.n);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

int dev_spmv_orig(Plan &P, const double *x, double *y) {
  int blocks = std::max(1, std::min((P.n + 7) / 8, 8192));
  k_spmv_orig<<<blocks, 256, 0, P.stream>>>(P.n, P.d_Rp, P.d_Rj, P.d_Rx, x, y);
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

// ---- GMRES refinement (reference pmgmres_ldlt_auto, src/gmres/mgmres.cpp:1015-1211)
namespace {
struct Gm {
  Plan &P;
  double *part;
  explicit Gm(Plan &p) : P(p), part(p.d_scal + 64) {}
  // dot into device slot, returns host value
  int dot(const double *a, const double *b, int slot, double &out) {
    k_dot_partial<<<DOT_BLOCKS, 256, 0, P.stream>>>(P.n, a, b, part);
    P.nlaunch++;
    k_dot_final<<<1, 256, 0, P.stream>>>(part, DOT_BLOCKS, P.d_scal + slot);
    P.nlaunch++;
    NQG_CUDA(cudaMemcpyAsync(&out, P.d_scal + slot, sizeof(double), cudaMemcpyDeviceToHost, P.stream));
    NQG_CUDA(cudaStreamSynchronize(P.stream));
    return NQG_OK;
  }
  int set_slot(int slot, double v) {
    NQG_CUDA(cudaMemcpyAsync(P.d_scal + slot, &v, sizeof(double), cudaMemcpyHostToDevice, P.stream));
    NQG_CUDA(cudaStreamSynchronize(P.stream));
    return NQG_OK;
  }
};
}  // namespace

// x_ord: initial solution in, refined solution out; b_ord: ordered rhs.
static int gmres_refine(Plan &P, double *x, const double *b, int &itr_used, double &rho_out) {
  const int n = P.n;
  const int itr_max = P.set.req_ref_iter, mr = P.set.max_inner_iter;
  itr_used = 0;
  rho_out = 0.0;
  if (itr_max <= 0 || mr <= 0) return NQG_OK;
  if (mr > P.mr_cap) return NQG_ERR_SIZE;
  const double delta = 1.0e-03;
  const double tol_abs = P.set.tol_abs, tol_rel = P.set.tol_rel;
  Gm g(P);
  double *r = P.d_r;
  double *V = P.d_V;
  std::vector<double> c(mr + 1), s(mr + 1), gg(mr + 1), y(mr + 1);
  std::vector<std::vector<double>> h(mr + 1, std::vector<double>(mr, 0.0));
  double rho = 0.0, rho_tol = 0.0;
  int rc;
  for (int itr = 0; itr < itr_max; ++itr) {
    if ((rc = dev_spmv_ord(P, x, r))) return rc;
    k_sub<<<grid_for(n), 256, 0, P.stream>>>(n, b, r);
    P.nlaunch++;
    if ((rc = dev_ldlt_solve_ord(P, r))) return rc;
    double rr;
    if ((rc = g.dot(r, r, 0, rr))) return rc;
    rho = std::sqrt(rr);
    rho_out = rho;
    if (rho < tol_abs) return NQG_OK;
    if (itr == 0) rho_tol = rho * tol_rel;
    if ((rc = g.set_slot(1, rho))) return rc;
    k_scale_div<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 1, r, V);
    P.nlaunch++;
    gg[0] = rho;
    for (int i = 1; i <= mr; ++i) gg[i] = 0.0;
    for (auto &row : h) std::fill(row.begin(), row.end(), 0.0);
    int k_copy = 0;
    for (int k = 0; k < mr; ++k) {
      k_copy = k;
      double *vk = V + (size_t)k * n, *vk1 = V + (size_t)(k + 1) * n;
      if ((rc = dev_spmv_ord(P, vk, vk1))) return rc;
      if ((rc = dev_ldlt_solve_ord(P, vk1))) return rc;
      double av2;
      if ((rc = g.dot(vk1, vk1, 0, av2))) return rc;
      const double av = std::sqrt(av2);
      for (int j = 0; j <= k; ++j) {
        double hj;
        if ((rc = g.dot(vk1, V + (size_t)j * n, 2, hj))) return rc;
        h[j][k] = hj;
        k_axpy<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 2, -1.0, V + (size_t)j * n, vk1);
        P.nlaunch++;
      }
      double hn2;
      if ((rc = g.dot(vk1, vk1, 0, hn2))) return rc;
      h[k + 1][k] = std::sqrt(hn2);
      if ((av + delta * h[k + 1][k]) == av) {
        for (int j = 0; j < k + 1; ++j) {
          double ht;
          if ((rc = g.dot(vk1, V + (size_t)j * n, 2, ht))) return rc;
          h[j][k] = h[j][k] + ht;
          k_axpy<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 2, -1.0, V + (size_t)j * n, vk1);
          P.nlaunch++;
        }
        if ((rc = g.dot(vk1, vk1, 0, hn2))) return rc;
        h[k + 1][k] = std::sqrt(hn2);
      }
      if (h[k + 1][k] != 0.0) {
        if ((rc = g.set_slot(1, h[k + 1][k]))) return rc;
        k_scale_div<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 1, vk1, vk1);
        P.nlaunch++;
      }
      if (0 < k) {
        for (int i = 0; i < k + 2; ++i) y[i] = h[i][k];
        for (int j = 0; j < k; ++j) {  // Givens rotations of the previous steps
          double g1 = c[j] * y[j] - s[j] * y[j + 1];
          double g2 = s[j] * y[j] + c[j] * y[j + 1];
          y[j] = g1;
          y[j + 1] = g2;
        }
        for (int i = 0; i < k + 2; ++i) h[i][k] = y[i];
      }
      const double mu = std::sqrt(h[k][k] * h[k][k] + h[k + 1][k] * h[k + 1][k]);
      if (mu == 0) return NQG_OK;
      c[k] = h[k][k] / mu;
      s[k] = -h[k + 1][k] / mu;
      h[k][k] = c[k] * h[k][k] - s[k] * h[k + 1][k];
      h[k + 1][k] = 0.0;
      {
        double g1 = c[k] * gg[k] - s[k] * gg[k + 1];
        double g2 = s[k] * gg[k] + c[k] * gg[k + 1];
        gg[k] = g1;
        gg[k + 1] = g2;
      }
      rho = std::fabs(gg[k + 1]);
      rho_out = rho;
      itr_used = itr_used + 1;
      if (rho <= rho_tol && rho <= tol_abs) break;
    }
    int k = k_copy;
    if (h[k][k] == 0) return NQG_OK;
    y[k] = gg[k] / h[k][k];
    for (int i = k - 1; 0 <= i; i--) {
      y[i] = gg[i];
      for (int j = i + 1; j < k + 1; j++) y[i] = y[i] - h[i][j] * y[j];
      y[i] = y[i] / h[i][i];
    }
    NQG_CUDA(cudaMemcpyAsync(P.d_scal + 8, y.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, P.stream));
    k_update_x<<<grid_for(n), 256, 0, P.stream>>>(n, k + 1, V, P.d_scal + 8, x);
    P.nlaunch++;
    NQG_CUDA(cudaGetLastError());
    if (rho <= rho_tol && rho <= tol_abs) break;
  }
  return NQG_OK;
}

// Flexible GMRES (right preconditioning; Saad, SIAM J. Sci. Comput. 14 (1993))
// around FP32 triangular solves.  z_k = M^-1 v_k is kept, the next Arnoldi
// vector comes from A z_k in FP64, so the minimised residual is b - A x
// itself: the rounding of the FP32 solves slows convergence at most, it does
// not cap the attainable accuracy as it does for the left-preconditioned
// loop.  Restarts, inner steps, reorthogonalisation test and stopping rule
// are those of gmres_refine.
static int fgmres_refine(Plan &P, double *x, const double *b, int &itr_used, double &rho_out) {
  const int n = P.n;
  const int itr_max = P.set.req_ref_iter, mr = P.set.max_inner_iter;
  itr_used = 0;
  rho_out = 0.0;
  if (itr_max <= 0 || mr <= 0) return NQG_OK;
  if (mr > P.mr_cap || !P.d_Z) return NQG_ERR_SIZE;
  const double delta = 1.0e-03;
  const double tol_abs = P.set.tol_abs, tol_rel = P.set.tol_rel;
  Gm g(P);
  double *r = P.d_r;
  double *V = P.d_V;
  float *Z = P.d_Z;
  std::vector<double> c(mr + 1), s(mr + 1), gg(mr + 1), y(mr + 1);
  std::vector<std::vector<double>> h(mr + 1, std::vector<double>(mr, 0.0));
  double rho = 0.0, rho_tol = 0.0;
  int rc;
  for (int itr = 0; itr < itr_max; ++itr) {
    if ((rc = dev_spmv_ord(P, x, r))) return rc;
    k_sub<<<grid_for(n), 256, 0, P.stream>>>(n, b, r);
    P.nlaunch++;
    double rr;
    if ((rc = g.dot(r, r, 0, rr))) return rc;
    rho = std::sqrt(rr);
    rho_out = rho;
    if (rho < tol_abs) return NQG_OK;
    if (itr == 0) rho_tol = rho * tol_rel;
    if ((rc = g.set_slot(1, rho))) return rc;
    k_scale_div<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 1, r, V);
    P.nlaunch++;
    gg[0] = rho;
    for (int i = 1; i <= mr; ++i) gg[i] = 0.0;
    for (auto &row : h) std::fill(row.begin(), row.end(), 0.0);
    int k_copy = 0;
    for (int k = 0; k < mr; ++k) {
      k_copy = k;
      double *vk = V + (size_t)k * n, *vk1 = V + (size_t)(k + 1) * n;
      float *zk = Z + (size_t)k * n;
      k_narrow<<<grid_for(n), 256, 0, P.stream>>>(n, vk, zk);
      P.nlaunch++;
      if ((rc = ldlt_solve_impl<float, float>(P, zk))) return rc;
      k_widen<<<grid_for(n), 256, 0, P.stream>>>(n, zk, P.d_w);
      P.nlaunch++;
      if ((rc = dev_spmv_ord(P, P.d_w, vk1))) return rc;
      double av2;
      if ((rc = g.dot(vk1, vk1, 0, av2))) return rc;
      const double av = std::sqrt(av2);
      for (int j = 0; j <= k; ++j) {
        double hj;
        if ((rc = g.dot(vk1, V + (size_t)j * n, 2, hj))) return rc;
        h[j][k] = hj;
        k_axpy<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 2, -1.0, V + (size_t)j * n, vk1);
        P.nlaunch++;
      }
      double hn2;
      if ((rc = g.dot(vk1, vk1, 0, hn2))) return rc;
      h[k + 1][k] = std::sqrt(hn2);
      if ((av + delta * h[k + 1][k]) == av) {
        for (int j = 0; j < k + 1; ++j) {
          double ht;
          if ((rc = g.dot(vk1, V + (size_t)j * n, 2, ht))) return rc;
          h[j][k] = h[j][k] + ht;
          k_axpy<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 2, -1.0, V + (size_t)j * n, vk1);
          P.nlaunch++;
        }
        if ((rc = g.dot(vk1, vk1, 0, hn2))) return rc;
        h[k + 1][k] = std::sqrt(hn2);
      }
      if (h[k + 1][k] != 0.0) {
        if ((rc = g.set_slot(1, h[k + 1][k]))) return rc;
        k_scale_div<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_scal + 1, vk1, vk1);
        P.nlaunch++;
      }
      if (0 < k) {
        for (int i = 0; i < k + 2; ++i) y[i] = h[i][k];
        for (int j = 0; j < k; ++j) {
          double g1 = c[j] * y[j] - s[j] * y[j + 1];
          double g2 = s[j] * y[j] + c[j] * y[j + 1];
          y[j] = g1;
          y[j + 1] = g2;
        }
        for (int i = 0; i < k + 2; ++i) h[i][k] = y[i];
      }
      const double mu = std::sqrt(h[k][k] * h[k][k] + h[k + 1][k] * h[k + 1][k]);
      if (mu == 0) return NQG_OK;
      c[k] = h[k][k] / mu;
      s[k] = -h[k + 1][k] / mu;
      h[k][k] = c[k] * h[k][k] - s[k] * h[k + 1][k];
      h[k + 1][k] = 0.0;
      {
        double g1 = c[k] * gg[k] - s[k] * gg[k + 1];
        double g2 = s[k] * gg[k] + c[k] * gg[k + 1];
        gg[k] = g1;
        gg[k + 1] = g2;
      }
      rho = std::fabs(gg[k + 1]);
      rho_out = rho;
      itr_used = itr_used + 1;
      if (rho <= rho_tol && rho <= tol_abs) break;
    }
    int k = k_copy;
    if (h[k][k] == 0) return NQG_OK;
    y[k] = gg[k] / h[k][k];
    for (int i = k - 1; 0 <= i; i--) {
      y[i] = gg[i];
      for (int j = i + 1; j < k + 1; j++) y[i] = y[i] - h[i][j] * y[j];
      y[i] = y[i] / h[i][i];
    }
    NQG_CUDA(cudaMemcpyAsync(P.d_scal + 8, y.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, P.stream));
    k_update_x_f<<<grid_for(n), 256, 0, P.stream>>>(n, k + 1, Z, P.d_scal + 8, x);
    P.nlaunch++;
    NQG_CUDA(cudaGetLastError());
    if (rho <= rho_tol && rho <= tol_abs) break;
  }
  return NQG_OK;
}

int dev_solve(Plan &P, const double *d_rhs, double *d_x) {
  const int n = P.n;
  int rc;
  // x_ord = rhs[perm]; b_ord = rhs[perm]
  k_gather<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_perm, d_rhs, P.d_bo);
  P.nlaunch++;
  NQG_CUDA(cudaMemcpyAsync(P.d_xo, P.d_bo, n * sizeof(double), cudaMemcpyDeviceToDevice, P.stream));
  if ((rc = dev_ldlt_solve_ord(P, P.d_xo))) return rc;
  int used = 0;
  double rho = 0;
  const bool flex = P.set.precision == NQG_FP32 && P.set.solve_precision == NQG_FP32;
  if ((rc = flex ? fgmres_refine(P, P.d_xo, P.d_bo, used, rho) : gmres_refine(P, P.d_xo, P.d_bo, used, rho)))
    return rc;
  P.tm.num_ref_iter = used;
  P.tm.last_residual = rho;
  k_scatter<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_perm, P.d_xo, d_x);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

// Refinement alone from x0 = rhs (reference iterative_ref_only,
// src/QP/linear_solver_wrapper.cpp:1406-1430): no initial triangular solve.
int dev_refine_only(Plan &P, const double *d_rhs, double *d_x) {
  const int n = P.n;
  int rc;
  k_gather<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_perm, d_rhs, P.d_bo);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  NQG_CUDA(cudaMemcpyAsync(P.d_xo, P.d_bo, n * sizeof(double), cudaMemcpyDeviceToDevice, P.stream));
  int used = 0;
  double rho = 0;
  const bool flex = P.set.precision == NQG_FP32 && P.set.solve_precision == NQG_FP32;
  if ((rc = flex ? fgmres_refine(P, P.d_xo, P.d_bo, used, rho) : gmres_refine(P, P.d_xo, P.d_bo, used, rho)))
    return rc;
  P.tm.num_ref_iter = used;
  P.tm.last_residual = rho;
  k_scatter<<<grid_for(n), 256, 0, P.stream>>>(n, P.d_perm, P.d_xo, d_x);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  return NQG_OK;
}

}  // namespace nqg
