// Allocation-free dense Bunch-Kaufman LDL^T (see nqg_dense_ldlt_noalloc in
// include/nasoq_gb300.h).
//
// All scratch lives in one file-scope device array, reserved when the
// library is loaded on a device and kept until the process exits.  Host code
// cannot use the array's name as a device address, so each call
// looks the address up with cudaGetSymbolAddress (with that device
// current) and every kernel receives pointers derived from it.  The lookup is
// repeated on every call (see scratch_for_current_device).
#include <cuda_runtime.h>

#include <mutex>

#include "coop.cuh"
#include "plan.hpp"

namespace nqg {
template <class T>
int factor_wide_raw(T *S, int nrow, int w, T *Dd, T *De, int *perm, T *Wb, WideCtl *ctl, int *status,
                    cudaStream_t st, int num_sms, int nb, int *pivoted);
}

namespace {

// Capacity of the shared scratch: panels of at most this many rows.
constexpr int NOALLOC_MAX_ROWS = 8192;
constexpr int NOALLOC_NB = 64;  // panel width; the W buffer holds nb+2 columns
constexpr size_t NOALLOC_CTL_BYTES = (sizeof(nqg::WideCtl) + 255) / 256 * 256;
constexpr size_t NOALLOC_STATUS_BYTES = 256;
constexpr size_t NOALLOC_W_BYTES = (size_t)NOALLOC_MAX_ROWS * (NOALLOC_NB + 2) * sizeof(double);
constexpr size_t NOALLOC_BYTES = NOALLOC_CTL_BYTES + NOALLOC_STATUS_BYTES + NOALLOC_W_BYTES;  // ~4.4 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
int g_sms[MAX_DEVICES] = {};

// Device address of the scratch array, looked up on every call with the
// caller's device current: a device reset or another context on the same
// ordinal reloads the module and may move the array, so an address kept from
// an earlier call could be stale.  The lookup allocates nothing.  The SM
// count of each device is kept after its first call.
int scratch_for_current_device(unsigned char **base, int *sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return NQG_ERR_CUDA;
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) return NQG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_sms[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return NQG_ERR_CUDA;
    g_sms[dev] = n;
  }
  *base = static_cast<unsigned char *>(p);
  *sms = g_sms[dev];
  return NQG_OK;
}

}  // namespace

extern "C" int nqg_dense_ldlt_noalloc(int nrow, int w, double *d_A, int lda, double *d_D, int *d_perm,
                                      void *stream) {
  if (nrow < 1 || w < 1 || w > nrow || !d_A || !d_D || !d_perm || lda != nrow) return NQG_ERR_ARG;
  if (nrow > NOALLOC_MAX_ROWS) return NQG_ERR_SIZE;
  unsigned char *base = nullptr;
  int sms = 0;
  int rc = scratch_for_current_device(&base, &sms);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto *ctl = reinterpret_cast<nqg::WideCtl *>(base);
  int *status = reinterpret_cast<int *>(base + NOALLOC_CTL_BYTES);
  double *Wb = reinterpret_cast<double *>(base + NOALLOC_CTL_BYTES + NOALLOC_STATUS_BYTES);
  // the array keeps the previous call's contents: clear what must start at zero
  if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return NQG_ERR_CUDA;
  if (cudaMemsetAsync(d_D, 0, (size_t)2 * w * sizeof(double), st) != cudaSuccess) return NQG_ERR_CUDA;
  rc = nqg::factor_wide_raw<double>(d_A, nrow, w, d_D, d_D + w, d_perm, Wb, ctl, status, st, sms, NOALLOC_NB,
                                    nullptr);
  if (rc) return rc;
  int hs = 0;
  if (cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return NQG_ERR_CUDA;
  if (hs & nqg::ST_TIMEOUT) return NQG_ERR_TIMEOUT;
  if (hs & nqg::ST_ZERO_PIVOT) return NQG_WARN_ZERO_PIVOT;
  return NQG_OK;
}
