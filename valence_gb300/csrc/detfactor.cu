/*
 * detfactor.cu -- batched determinant and inverse of small dense matrices,
 * the factorisation the energy path applies to every spin block of every
 * determinant pair (replacing givdr/givens_single, valence.F90:2067-2144,
 * givens.F90:230-262, whose product of the triangularised diagonal is the
 * determinant).  Exposed on its own for hosts that factorise overlap blocks
 * themselves, e.g. a first-order optimiser assembling H/S per substituted
 * orbital (valence.F90:527-844).
 *
 * One block per matrix: Gauss-Jordan elimination with partial pivoting on
 * the augmented [A | I] in a scratch area of n x 2n doubles per matrix.  A
 * pivot below 1e-7 of the matrix's largest entry marks the matrix singular:
 * its determinant is then taken by LU on a fresh copy and its inverse is
 * left zero.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/vsvb_gpu.h"

namespace {

constexpr int GJ_THREADS = 128;

__device__ double gj_block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    red[0] = m;
  }
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

/* W: this matrix's n x 2n scratch */
__device__ void gauss_jordan(const double *A, int n, double *W, double *det_out, double *inv_out, int *sing_out) {
  __shared__ double red[GJ_THREADS / 32];
  __shared__ int redi[GJ_THREADS / 32];
  __shared__ double sdet;
  __shared__ int ssing, spiv;
  const int n2 = 2 * n;
  double mx = 0.0;
  for (int t = threadIdx.x; t < n * n2; t += blockDim.x) {
    const int r = t / n2, c = t - r * n2;
    double v;
    if (c < n) {
      v = A[r * n + c];
      mx = fmax(mx, fabs(v));
    } else {
      v = (c - n == r) ? 1.0 : 0.0;
    }
    W[t] = v;
  }
  const double amax = gj_block_max(mx, red);
  if (threadIdx.x == 0) {
    sdet = 1.0;
    ssing = 0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      const double v = fabs(W[i * n2 + k]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = best;
      redi[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = -1.0;
      int p = k;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        if (red[w] > b || (red[w] == b && redi[w] < p)) {
          b = red[w];
          p = redi[w];
        }
      spiv = p;
      if (!(b > 1e-7 * amax)) ssing = 1;
    }
    __syncthreads();
    if (ssing) break;
    const int p = spiv;
    if (p != k)
      for (int j = threadIdx.x; j < n2; j += blockDim.x) {
        const double t = W[k * n2 + j];
        W[k * n2 + j] = W[p * n2 + j];
        W[p * n2 + j] = t;
      }
    __syncthreads();
    const double piv = W[k * n2 + k];
    if (threadIdx.x == 0) sdet *= (p != k ? -piv : piv);
    __syncthreads();
    for (int j = threadIdx.x; j < n2; j += blockDim.x) W[k * n2 + j] /= piv;
    __syncthreads();
    for (int t = threadIdx.x; t < n * n2; t += blockDim.x) {
      const int i = t / n2, j = t - i * n2;
      if (i != k && j != k) W[t] -= W[i * n2 + k] * W[k * n2 + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k) W[i * n2 + k] = 0.0;
    __syncthreads();
  }
  if (ssing) {
    if (threadIdx.x == 0) {
      double *M = W;
      for (int t = 0; t < n * n; ++t) M[t] = A[t];
      double det = 1.0;
      for (int k = 0; k < n && det != 0.0; ++k) {
        int p = k;
        double m = fabs(M[k * n + k]);
        for (int i = k + 1; i < n; ++i)
          if (fabs(M[i * n + k]) > m) {
            m = fabs(M[i * n + k]);
            p = i;
          }
        if (m == 0.0) {
          det = 0.0;
          break;
        }
        if (p != k) {
          for (int j = 0; j < n; ++j) {
            const double t = M[k * n + j];
            M[k * n + j] = M[p * n + j];
            M[p * n + j] = t;
          }
          det = -det;
        }
        det *= M[k * n + k];
        for (int i = k + 1; i < n; ++i) {
          const double f = M[i * n + k] / M[k * n + k];
          for (int j = k + 1; j < n; ++j) M[i * n + j] -= f * M[k * n + j];
        }
      }
      *det_out = det;
      *sing_out = 1;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) inv_out[t] = 0.0;
  } else {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int r = t / n, c = t - r * n;
      inv_out[t] = W[r * n2 + n + c];
    }
    if (threadIdx.x == 0) {
      *det_out = sdet;
      *sing_out = 0;
    }
  }
}

__global__ void det_factor_kernel(const double *A, int n, double *scratch, double *det, double *inv, int *sing) {
  const size_t m = blockIdx.x;
  gauss_jordan(A + m * n * n, n, scratch + m * 2 * (size_t)n * n, det + m, inv + m * n * n, sing + m);
}

}  // namespace

extern "C" int vsvb_det_factor(const double *a_dev, int n, int nmat, double *det_dev, double *inv_dev, int *sing_dev,
                               void *stream) {
  if (n < 1 || nmat < 0 || !a_dev || !det_dev || !inv_dev || !sing_dev) return VSVB_ERR_INPUT;
  if (nmat == 0) return VSVB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *scratch = nullptr;
  if (cudaMalloc(&scratch, sizeof(double) * 2 * (size_t)n * n * nmat) != cudaSuccess) return VSVB_ERR_NOMEM;
  det_factor_kernel<<<nmat, GJ_THREADS, 0, st>>>(a_dev, n, scratch, det_dev, inv_dev, sing_dev);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(scratch);
  return e == cudaSuccess ? VSVB_OK : VSVB_ERR_CUDA;
}

/*
 * Allocation-free variant.  Some callers cannot call cudaMalloc at the
 * moment they need a factorisation: a Fortran optimiser that runs inside a
 * host-side memory budget handed to it by another framework (PyTorch's
 * caching allocator owns the device pool, and a raw cudaMalloc would grow
 * or fragment it behind that allocator's back), or code running between
 * kernels of a larger asynchronous pipeline whose owner forbids device
 * allocation in that phase.  This entry point takes its scratch from a
 * fixed file-scope device array instead of allocating.
 *
 * Limits and behaviour:
 *  - the scratch holds VSVB_NOALLOC_SCRATCH_DOUBLES doubles (4 MiB) on every
 *    device that loads the library, for the life of the process; a call
 *    needs 2*n*n*nmat of them and is rejected with VSVB_ERR_TOO_LARGE beyond
 *    that;
 *  - the first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current and keeps it for the
 *    life of the process: a cudaDeviceReset may move the array, so the
 *    library must not be used across one;
 *  - every call synchronises its stream before returning, so none may be
 *    made while that stream is capturing a CUDA graph;
 *  - every call shares the one array, which keeps the previous call's
 *    contents (each call rewrites all the scratch it reads); calls whose
 *    work overlaps on the GPU race on it, so serialise them (one stream, or
 *    wait between calls);
 *  - no cudaMalloc, cudaFree or allocating library routine is called.
 */
#define VSVB_NOALLOC_SCRATCH_DOUBLES (1 << 19)

static __device__ __align__(256) double g_noalloc_scratch[VSVB_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
double *g_noalloc_addr[kMaxDevices] = {};
std::mutex g_noalloc_mu;
}  // namespace

extern "C" int vsvb_det_factor_noalloc(const double *a_dev, int n, int nmat, double *det_dev, double *inv_dev,
                                       int *sing_dev, void *stream) {
  if (n < 1 || nmat < 0 || !a_dev || !det_dev || !inv_dev || !sing_dev) return VSVB_ERR_INPUT;
  if ((double)2 * n * n * (double)nmat > (double)VSVB_NOALLOC_SCRATCH_DOUBLES) return VSVB_ERR_TOO_LARGE;
  if (nmat == 0) return VSVB_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VSVB_ERR_CUDA;
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void *addr = nullptr;
      if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) return VSVB_ERR_CUDA;
      g_noalloc_addr[dev] = static_cast<double *>(addr);
    }
    scratch = g_noalloc_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  det_factor_kernel<<<nmat, GJ_THREADS, 0, st>>>(a_dev, n, scratch, det_dev, inv_dev, sing_dev);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? VSVB_OK : VSVB_ERR_CUDA;
}
