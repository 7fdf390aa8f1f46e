// FCT_positivity for callers that cannot allocate device memory.
//
// The context-based entry points allocate their buffers with cudaMalloc when
// a context is created.  Some callers cannot do that: a host code that hands
// the library device buffers it manages itself through its own memory pool or
// a preallocated arena, a Fortran driver that maps its arrays to the device
// once and forbids further allocations, or code that must not grow the
// process's device footprint while other work is resident.  For those, this
// file provides FCT_positivity (SOURCES/fct.f90:5-42) as one call that takes
// device pointers for every input and output and keeps its only scratch
// array -- R^- per node -- in a fixed device array compiled into the library.
//
// Contract (also stated in include/swe_gpu.h):
//  * np must not exceed SWE_NOALLOC_MAX_NODES; larger sizes are rejected with
//    SWE_ERR_ARG before anything is launched.
//  * The scratch array is a file-scope __device__ array: every GPU that loads
//    the library holds SWE_NOALLOC_MAX_NODES doubles (8 MiB) until the process
//    exits, and every call shares it.  Calls whose kernels overlap on the GPU
//    (different streams, or different host threads) race on it; serialise
//    them.  The array keeps the previous call's contents; nothing in it needs
//    to start at zero because every R^-_i is written before it is read.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress while that device is current, once per device.
//  * Every call synchronises the caller's stream before it returns (to read
//    the column-check flag), so no call can be recorded into a CUDA graph.
//  * d_ia and d_ja must form a valid 1-based CSR structure of the caller's
//    d_mat / d_lij arrays (ia(1) = 1, non-decreasing).  Column indices are
//    checked on the device: a column outside 1..np is not read through, and
//    the call returns SWE_ERR_ARG (d_lij is then unspecified).
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/swe_gpu.h"

namespace {

static __device__ __align__(256) double g_rminus_scratch[SWE_NOALLOC_MAX_NODES];
// set by the kernels when the CSR structure is out of range (cleared per call)
static __device__ unsigned g_noalloc_bad;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};
unsigned* g_bad_addr[kMaxDevices] = {nullptr};

// R^-_i (fct.f90:15-30): P^- = -1e-15 + sum_{f_ij<0} f_ij in CSR order,
// R^- = min(Q^-/P^-, 1) with Q^- = 0 - unext, 0 where unext <= htiny.
__global__ void k_noalloc_rminus(int np, const int* __restrict__ ia, const double* __restrict__ unext,
                                 const double* __restrict__ mat, double htiny, double* __restrict__ rminus,
                                 unsigned* __restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    if ((i == 0 && ia[0] != 1) || ia[i + 1] < ia[i]) atomicOr(bad, 1u);
    double P = -1.e-15;
    for (int p = ia[i] - 1; p < ia[i + 1] - 1; p++) {
      const double f = mat[p];
      if (f < 0.0) P = P + f;
    }
    const double u = unext[i];
    double R = (0.0 - u) / P;
    R = R < 1.0 ? R : 1.0;
    if (u <= htiny) R = 0.0;
    rminus[i] = R;
  }
}

// l_ij = R^-_j if f_ij >= 0 else R^-_i (fct.f90:31-41)
// A column outside 1..np is flagged and not read through.
__global__ void k_noalloc_lij(int np, const int* __restrict__ ia, const int* __restrict__ ja,
                              const double* __restrict__ mat, const double* __restrict__ rminus,
                              double* __restrict__ lij, unsigned* __restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const double Ri = rminus[i];
    for (int p = ia[i] - 1; p < ia[i + 1] - 1; p++) {
      const int j = ja[p];
      if (j < 1 || j > np) {
        atomicOr(bad, 2u);
        continue;
      }
      lij[p] = (mat[p] >= 0.0) ? rminus[j - 1] : Ri;
    }
  }
}

int scratch_address(double** out, unsigned** bad) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SWE_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    void* q = nullptr;
    if (cudaGetSymbolAddress(&p, g_rminus_scratch) != cudaSuccess || !p) return SWE_ERR_CUDA;
    if (cudaGetSymbolAddress(&q, g_noalloc_bad) != cudaSuccess || !q) return SWE_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<double*>(p);
    g_bad_addr[dev] = static_cast<unsigned*>(q);
  }
  *out = g_scratch_addr[dev];
  *bad = g_bad_addr[dev];
  return SWE_OK;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int swe_fct_positivity_noalloc(
    int np, const int* d_ia, const int* d_ja, const double* d_unext, const double* d_mat, double htiny,
    double* d_lij, void* stream) {
  if (np <= 0 || !d_ia || !d_ja || !d_unext || !d_mat || !d_lij) return SWE_ERR_ARG;
  if (np > SWE_NOALLOC_MAX_NODES) return SWE_ERR_ARG;
  double* rminus = nullptr;
  unsigned* bad = nullptr;
  int rc = scratch_address(&rminus, &bad);
  if (rc) return rc;
  // an error left by earlier, unrelated launches is not this call's
  (void)cudaGetLastError();
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int bs = 256;
  const int nb = (np + bs - 1) / bs;
  unsigned flag = 0;
  if (cudaMemsetAsync(bad, 0, sizeof(unsigned), s) != cudaSuccess) return SWE_ERR_CUDA;
  k_noalloc_rminus<<<nb, bs, 0, s>>>(np, d_ia, d_unext, d_mat, htiny, rminus, bad);
  k_noalloc_lij<<<nb, bs, 0, s>>>(np, d_ia, d_ja, d_mat, rminus, d_lij, bad);
  if (cudaGetLastError() != cudaSuccess) return SWE_ERR_CUDA;
  if (cudaMemcpyAsync(&flag, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SWE_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SWE_ERR_CUDA;
  return flag ? SWE_ERR_ARG : SWE_OK;
}
