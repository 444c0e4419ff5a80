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

#include "coop.cuh"
#include "plan.hpp"

namespace nqg {

namespace {

constexpr int WP_THREADS = 256;

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
      double x = pv[g];
      int xi = pi[g];
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

// One panel: columns c = k0 .. (at most k0+nb, one more for a final 2x2).
template <class T>
__global__ void __launch_bounds__(WP_THREADS) k_wide_panel(T *S, int nrow, int w, int k0, int nb, T *Wb, int ldw,
                                                           T *Dd, T *De, int *perm, WideCtl *ctl, int *status) {
  __shared__ T wrow[128];
  const T alpha = (T)((1.0 + sqrt(17.0)) / 8.0);
  const int G = gridDim.x;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int TT = G * blockDim.x;
  // Every row keeps the same owner thread in every step (r % TT == gt), so a
  // thread reads back only the L entries it wrote itself between barriers.
  auto first_row = [&](int lo) { return lo + (int)(((long long)gt - lo % TT + TT) % TT); };
  int j = 0;
  int parity = 0;
  while (j < nb && k0 + j < w) {
    const int c = k0 + j;
    // ---- A: updated column c into W(:, j), rows [c, nrow)
    for (int t = threadIdx.x; t < j; t += blockDim.x) wrow[t] = Wb[(size_t)t * ldw + c];
    __syncthreads();
    T cv = T(-1);
    int ci = -1;
    for (int r = first_row(c); r < nrow; r += TT) {
      T acc = S[r + (size_t)c * nrow];
      for (int t = 0; t < j; ++t) acc -= S[r + (size_t)(k0 + t) * nrow] * wrow[t];
      Wb[(size_t)j * ldw + r] = acc;
      if (r > c && r < w) {
        T a = tabs_w(acc);
        if (ci < 0 || a > cv) {
          cv = a;
          ci = r;
        }
      }
    }
    cta_argmax(cv, ci);
    if (threadIdx.x == 0) {
      ctl->cval[parity][blockIdx.x] = (double)cv;
      ctl->cidx[parity][blockIdx.x] = ci;
    }
    if (!grid_sync(ctl, status)) return;
    T colmax;
    int imax;
    reduce_partials(ctl->cval[parity], ctl->cidx[parity], G, colmax, imax);
    if (imax < 0) colmax = T(0);
    const T absakk = tabs_w(Wb[(size_t)j * ldw + c]);
    int kp = c, kstep = 1;
    bool zero = false;
    if ((absakk >= colmax ? absakk : colmax) == T(0) || absakk != absakk) {
      zero = true;
    } else if (absakk < alpha * colmax) {
      // ---- B: updated column imax into W(:, j+1) and its off-diagonal max
      for (int t = threadIdx.x; t < j; t += blockDim.x) wrow[t] = Wb[(size_t)t * ldw + imax];
      __syncthreads();
      T rv = T(-1);
      int ri = -1;
      for (int r = first_row(c); r < nrow; r += TT) {
        T acc = r < imax ? S[imax + (size_t)r * nrow] : S[r + (size_t)imax * nrow];
        for (int t = 0; t < j; ++t) acc -= S[r + (size_t)(k0 + t) * nrow] * wrow[t];
        Wb[(size_t)(j + 1) * ldw + r] = acc;
        if (r < w && r != imax) {
          T a = tabs_w(acc);
          if (ri < 0 || a > rv) {
            rv = a;
            ri = r;
          }
        }
      }
      cta_argmax(rv, ri);
      if (threadIdx.x == 0) {
        ctl->rval[parity][blockIdx.x] = (double)rv;
        ctl->ridx[parity][blockIdx.x] = ri;
      }
      if (!grid_sync(ctl, status)) return;
      T rowmax;
      int rdummy;
      reduce_partials(ctl->rval[parity], ctl->ridx[parity], G, rowmax, rdummy);
      const T diag_imax = tabs_w(Wb[(size_t)(j + 1) * ldw + imax]);
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
        if (copycol && r != kk && r != kp) Wb[(size_t)j * ldw + r] = Wb[(size_t)(j + 1) * ldw + r];
        if (r > kp) {
          T t = S[r + (size_t)kk * nrow];
          S[r + (size_t)kk * nrow] = S[r + (size_t)kp * nrow];
          S[r + (size_t)kp * nrow] = t;
        } else if (r > kk && r < kp) {
          T t = S[r + (size_t)kk * nrow];
          S[r + (size_t)kk * nrow] = S[kp + (size_t)r * nrow];
          S[kp + (size_t)r * nrow] = t;
        }
      }
      for (int col = gt; col < kk; col += TT) {  // rows kk, kp of all finished columns
        T t = S[kk + (size_t)col * nrow];
        S[kk + (size_t)col * nrow] = S[kp + (size_t)col * nrow];
        S[kp + (size_t)col * nrow] = t;
      }
      if (gt == 0) {
        T t = S[kk + (size_t)kk * nrow];
        S[kk + (size_t)kk * nrow] = S[kp + (size_t)kp * nrow];
        S[kp + (size_t)kp * nrow] = t;
        int pt = perm[kk - 0];
        perm[kk] = perm[kp];
        perm[kp] = pt;
        if (copycol) {
          T a1 = Wb[(size_t)(j + 1) * ldw + kp], a2 = Wb[(size_t)(j + 1) * ldw + kk];
          Wb[(size_t)j * ldw + kk] = a1;
          Wb[(size_t)j * ldw + kp] = a2;
          for (int t2 = 0; t2 < j; ++t2) {
            T x = Wb[(size_t)t2 * ldw + kk];
            Wb[(size_t)t2 * ldw + kk] = Wb[(size_t)t2 * ldw + kp];
            Wb[(size_t)t2 * ldw + kp] = x;
          }
        } else {
          for (int t2 = 0; t2 <= j + 1; ++t2) {
            T x = Wb[(size_t)t2 * ldw + kk];
            Wb[(size_t)t2 * ldw + kk] = Wb[(size_t)t2 * ldw + kp];
            Wb[(size_t)t2 * ldw + kp] = x;
          }
        }
        ctl->pivoted = 1;
      }
      if (!grid_sync(ctl, status)) return;
    }
    // ---- D: L column(s) from W, D entries
    if (kstep == 1) {
      const T d = Wb[(size_t)j * ldw + c];
      if (!zero) {
        const T r1 = T(1) / d;
        for (int r = first_row(c + 1); r < nrow; r += TT) S[r + (size_t)c * nrow] = Wb[(size_t)j * ldw + r] * r1;
      } else if (gt == 0) {
        atomicOr(status, ST_ZERO_PIVOT);
      }
      if (gt == 0) {
        S[c + (size_t)c * nrow] = T(1);
        Dd[c] = d;
        De[c] = T(0);
      }
    } else {
      const T D11 = Wb[(size_t)j * ldw + c], D21 = Wb[(size_t)j * ldw + c + 1];
      const T D22 = Wb[(size_t)(j + 1) * ldw + c + 1];
      T d21 = D21;
      const T d11 = D22 / d21, d22 = D11 / d21;
      const T tt = T(1) / (d11 * d22 - T(1));
      d21 = tt / d21;
      for (int r = first_row(c + 2); r < nrow; r += TT) {
        const T wk = Wb[(size_t)j * ldw + r], wk1 = Wb[(size_t)(j + 1) * ldw + r];
        S[r + (size_t)c * nrow] = d21 * (d11 * wk - wk1);
        S[r + (size_t)(c + 1) * nrow] = d21 * (d22 * wk1 - wk);
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
    parity ^= 1;
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

template <class T> __global__ void k_wide_init_perm(int *perm, int w) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < w; m += gridDim.x * blockDim.x) perm[m] = m;
}

template <class T> __global__ void k_wide_zero_upper(T *S, int nrow, int w) {
  // entries above the diagonal of the diagonal block stay 0
  for (int c = blockIdx.x; c < w; c += gridDim.x)
    for (int r = threadIdx.x; r < c; r += blockDim.x) S[r + (size_t)c * nrow] = T(0);
}

}  // namespace

// Host driver for one wide supernode s.  Scratch: Wb (nrow x (nb+2)), ctl.
template <class T>
int factor_wide(Plan &P, int s, T *L, T *Dg, int nb, T *Wb, WideCtl *ctl, int num_sms) {
  cudaStream_t st = P.stream;
  const int c0 = P.sym.super[s], w = P.sym.super[s + 1] - c0;
  const int nrow = (int)(P.sym.lpi[s + 1] - P.sym.lpi[s]);
  T *S = L + P.sym.lpx[s];
  const int n = P.n;
  int *perm = P.d_locperm + c0;
  k_wide_init_perm<T><<<(w + 255) / 256, 256, 0, st>>>(perm, w);
  P.nlaunch++;
  NQG_CUDA(cudaMemsetAsync(ctl, 0, sizeof(WideCtl), st));
  int occ = 0;
  NQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_wide_panel<T>, WP_THREADS, 0));
  const int maxG = std::max(1, std::min(occ * num_sms, 1024));
  T *Dd = Dg + c0, *De = Dg + n + c0;
  int *status = P.d_status;
  int k0 = 0;
  while (k0 < w) {
    int rows_left = nrow - k0;
    int G = std::max(1, std::min(maxG, std::min(num_sms, (rows_left + 511) / 512)));
    int kb_want = std::min(nb, w - k0);
    void *args[] = {&S, (void *)&nrow, (void *)&w, &k0, &kb_want, &Wb, (void *)&nrow, &Dd, &De, &perm, &ctl, &status};
    cudaEvent_t e0 = P.prof_begin();
    NQG_CUDA(cudaLaunchCooperativeKernel((void *)k_wide_panel<T>, dim3(G), dim3(WP_THREADS), args, 0, st));
    P.nlaunch++;
    int kb = 0;
    NQG_CUDA(cudaMemcpyAsync(&kb, &ctl->kb, sizeof(int), cudaMemcpyDeviceToHost, st));
    NQG_CUDA(cudaStreamSynchronize(st));
    int abort = 0;
    NQG_CUDA(cudaMemcpy(&abort, &ctl->abort, sizeof(int), cudaMemcpyDeviceToHost));
    if (abort || kb <= 0) return NQG_ERR_TIMEOUT;
    const int k1 = k0 + kb;
    {
      // panel: column GEMVs (2 * rows * j) and the L column scaling
      double fl = 0;
      for (int j = 0; j < kb; ++j) fl += 2.0 * (nrow - (k0 + j)) * (j + 1);
      P.prof_end(NQG_K_WIDE_PANEL, e0, fl, 0.0);
    }
    if (k1 < w) {
      cudaEvent_t e1 = P.prof_begin();
      if (sizeof(T) == 4) {
        constexpr int BM = 128, BN = 128;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 8, 8><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      } else {
        constexpr int BM = 64, BN = 64;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 4, 4><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      }
      P.nlaunch++;
      // useful multiply-adds: kb per entry of the lower trapezoid rows [k1,nrow) x cols [k1,w)
      const double cols = w - k1;
      const double entries = cols * (nrow - k1) - cols * (cols - 1) / 2.0;
      P.prof_end(NQG_K_WIDE_TRAILING, e1, 2.0 * kb * entries, 0.0);
      NQG_CUDA(cudaGetLastError());
    }
    k0 = k1;
  }
  k_wide_zero_upper<T><<<std::min(w, 1024), 128, 0, st>>>(S, nrow, w);
  P.nlaunch++;
  NQG_CUDA(cudaGetLastError());
  int piv = 0;
  NQG_CUDA(cudaMemcpyAsync(&piv, &ctl->pivoted, sizeof(int), cudaMemcpyDeviceToHost, st));
  NQG_CUDA(cudaStreamSynchronize(st));
  uint8_t pv = piv ? 1 : 0;
  NQG_CUDA(cudaMemcpyAsync(P.d_pivoted + s, &pv, 1, cudaMemcpyHostToDevice, st));
  NQG_CUDA(cudaStreamSynchronize(st));
  return NQG_OK;
}

size_t wide_ctl_bytes() { return sizeof(WideCtl); }

// Same panel / trailing-update sequence as factor_wide, on caller-provided
// buffers (values S, D, E, perm) and caller-provided scratch (Wb, ctl,
// status); used by the allocation-free dense entry point.
template <class T>
int factor_wide_raw(T *S, int nrow, int w, T *Dd, T *De, int *perm, T *Wb, WideCtl *ctl, int *status,
                    cudaStream_t st, int num_sms, int nb, int *pivoted) {
  k_wide_init_perm<T><<<(w + 255) / 256, 256, 0, st>>>(perm, w);
  if (cudaMemsetAsync(ctl, 0, sizeof(WideCtl), st) != cudaSuccess) return NQG_ERR_CUDA;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_wide_panel<T>, WP_THREADS, 0) != cudaSuccess)
    return NQG_ERR_CUDA;
  const int maxG = std::max(1, std::min(occ * num_sms, 1024));
  int k0 = 0;
  while (k0 < w) {
    int rows_left = nrow - k0;
    int G = std::max(1, std::min(maxG, std::min(num_sms, (rows_left + 511) / 512)));
    int kb_want = std::min(nb, w - k0);
    int ldw = nrow;
    void *args[] = {&S, &nrow, &w, &k0, &kb_want, &Wb, &ldw, &Dd, &De, &perm, &ctl, &status};
    if (cudaLaunchCooperativeKernel((void *)k_wide_panel<T>, dim3(G), dim3(WP_THREADS), args, 0, st) != cudaSuccess)
      return NQG_ERR_CUDA;
    int kb = 0, abort = 0;
    if (cudaMemcpyAsync(&kb, &ctl->kb, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&abort, &ctl->abort, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return NQG_ERR_CUDA;
    if (abort || kb <= 0) return NQG_ERR_TIMEOUT;
    const int k1 = k0 + kb;
    if (k1 < w) {
      if (sizeof(T) == 4) {
        constexpr int BM = 128, BN = 128;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 8, 8><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      } else {
        constexpr int BM = 64, BN = 64;
        int tm = (nrow - k1 + BM - 1) / BM, tn = (w - k1 + BN - 1) / BN;
        k_wide_trailing<T, BM, BN, 4, 4><<<tm * tn, 256, 0, st>>>(S, nrow, w, k0, kb, Wb, nrow, tn);
      }
      if (cudaGetLastError() != cudaSuccess) return NQG_ERR_CUDA;
    }
    k0 = k1;
  }
  k_wide_zero_upper<T><<<std::min(w, 1024), 128, 0, st>>>(S, nrow, w);
  int piv = 0;
  if (cudaMemcpyAsync(&piv, &ctl->pivoted, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return NQG_ERR_CUDA;
  if (pivoted) *pivoted = piv;
  return NQG_OK;
}

template int factor_wide_raw<double>(double *, int, int, double *, double *, int *, double *, WideCtl *, int *,
                                     cudaStream_t, int, int, int *);

template int factor_wide<float>(Plan &, int, float *, float *, int, float *, WideCtl *, int);
template int factor_wide<double>(Plan &, int, double *, double *, int, double *, WideCtl *, int);

}  // namespace nqg
