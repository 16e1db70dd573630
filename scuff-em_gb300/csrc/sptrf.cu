// sptrf.cu -- symmetric matrices in packed storage: Bunch-Kaufman
// factorisation A = U D U^T and solves, on the GPU.
//
// Replaces the LHM_SYMMETRIC branches of HMatrix::LUFactorize / LUSolve
// (libs/libhmat/LBWrappers.cc:151-171, 175-236), which call LAPACK's
// dsptrf_/zsptrf_ and dsptrs_/zsptrs_ with UPLO = 'U', and the packed
// destinations of AssembleBEMMatrixBlock (scuff-cas3D keeps its diagonal T
// blocks as LHM_REAL + LHM_SYMMETRIC, applications/scuff-cas3D/
// CreateSC3Data.cc:110).
//
// Storage (HMatrix.cc:333 and LAPACK's 'U' packed format): the upper
// triangle by columns, entry (i, j), i <= j, at i + j (j + 1) / 2.  Complex
// matrices are complex symmetric (A = A^T, no conjugation), as zsptrf.
//
// Factorisation: LAPACK's published Bunch-Kaufman partial pivoting for the
// upper packed form, column k from N-1 down to 0, with its pivot rule
// (alpha = (1 + sqrt 17) / 8; |.| = |Re| + |Im| for complex entries; first
// index of the largest magnitude), its interchange of rows and columns kk and
// kp of the leading block, its rank-1 / rank-2 updates, the multipliers
// stored in place, and its 1-based pivot codes (negative pairs for 2 x 2
// blocks).  One cooperative kernel runs all columns: per column a grid-wide
// argmax, the pivot decision (taken by every block from the same partial
// results, so no broadcast is needed), the interchange, and the update of the
// leading block with one warp per column (packed columns are contiguous).
// The multipliers of a column are stored while the next column's argmax
// runs, since they touch columns the next step never reads.
//
// Solve: dsptrs' two passes (U D then U^T), one warp per right-hand side.
#include <cooperative_groups.h>
#include <climits>
#include <cmath>
#include <algorithm>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {
namespace cg = cooperative_groups;

namespace {

constexpr int SP_THREADS = 256;

__device__ __forceinline__ size_t pidx(int i, int j) { return (size_t)i + (size_t)j * (size_t)(j + 1) / 2; }

__device__ __forceinline__ double sp_mag(double x) { return fabs(x); }
__device__ __forceinline__ double sp_mag(cx<double> z) { return fabs(z.re) + fabs(z.im); }
__device__ __forceinline__ double sp_neg(double x) { return -x; }
__device__ __forceinline__ cx<double> sp_neg(cx<double> z) { return mk(-z.re, -z.im); }
__device__ __forceinline__ double sp_div(double a, double b) { return a / b; }
// complex quotient by Smith's scaling (no overflow for moderate operands)
__device__ __forceinline__ cx<double> sp_div(cx<double> a, cx<double> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return mk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  }
  const double r = b.re / b.im, d = b.im + b.re * r;
  return mk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__device__ __forceinline__ double shfl_xor_any(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ cx<double> shfl_xor_any(cx<double> v, int o) {
  return mk(__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o));
}
template <typename T> __device__ __forceinline__ T sp_zero();
template <> __device__ __forceinline__ double sp_zero<double>() { return 0.0; }
template <> __device__ __forceinline__ cx<double> sp_zero<cx<double>>() { return mk(0.0, 0.0); }
template <typename T> __device__ __forceinline__ T sp_one();
template <> __device__ __forceinline__ double sp_one<double>() { return 1.0; }
template <> __device__ __forceinline__ cx<double> sp_one<cx<double>>() { return mk(1.0, 0.0); }

struct Best {
  double v;
  int i;
};
// larger magnitude wins; equal magnitudes go to the smaller index (IDAMAX)
__device__ __forceinline__ Best better(Best a, Best b) { return (b.v > a.v || (b.v == a.v && b.i < a.i)) ? b : a; }

__device__ Best block_best(Best b, Best* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, c);
  }
  if (lane == 0) sh[wid] = b;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = better(b, sh[w]);
  __syncthreads();
  return b;  // valid in thread 0
}

__device__ double block_max(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = fmax(v, sh[w]);
  __syncthreads();
  return v;  // valid in thread 0
}

template <typename T>
__device__ __forceinline__ void sp_swap(T* AP, size_t a, size_t b) {
  const T t = AP[a];
  AP[a] = AP[b];
  AP[b] = t;
}

// Multipliers of column kc (1 x 1 pivot: column scaled by r1) or of columns
// kc-1, kc (2 x 2 pivot: WK, WKM1 from the columns' current values).
template <typename T>
__device__ void store_multipliers(T* AP, int kind, int kc, T r1, T d11, T d22, T d12, int gtid, int gthreads) {
  if (kind == 1) {
    for (int i = gtid; i < kc; i += gthreads) AP[pidx(i, kc)] = r1 * AP[pidx(i, kc)];
  } else if (kind == 2) {
    for (int j = gtid; j < kc - 1; j += gthreads) {
      const T a = AP[pidx(j, kc - 1)], b = AP[pidx(j, kc)];
      AP[pidx(j, kc)] = d12 * (d22 * b - a);      // WK
      AP[pidx(j, kc - 1)] = d12 * (d11 * a - b);  // WKM1
    }
  }
}

// pv: 2 * gridDim.x partial maxima (double-buffered by column parity),
// pi: their indices, pr: gridDim.x partial row maxima
template <typename T>
__global__ void __launch_bounds__(SP_THREADS) sptrf_kernel(T* AP, int N, int* ipiv, int* info, double* pv, int* pi,
                                                           double* pr) {
  cg::grid_group grid = cg::this_grid();
  __shared__ Best shb[SP_THREADS / 32];
  __shared__ double shd[SP_THREADS / 32];
  __shared__ Best s_col;
  __shared__ double s_row;
  const double alpha = (1.0 + sqrt(17.0)) * 0.125;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const int gwarp = gtid >> 5, gwarps = gthreads >> 5;
  const T one = sp_one<T>();
  int kind = 0, kc = -1;
  T r1 = one, d11 = one, d22 = one, d12 = one;
  int parity = 0;
  int k = N - 1;
  while (k >= 0) {
    // ---- phase A: the previous column's multipliers; argmax over column k above the diagonal
    store_multipliers(AP, kind, kc, r1, d11, d22, d12, gtid, gthreads);
    kind = 0;
    // every input of the pivot decision is read before a grid barrier that
    // precedes the first write of this column step (another block may be
    // interchanging entries once it is past that barrier)
    const double absakk = sp_mag(AP[pidx(k, k)]);
    Best b = {-1.0, INT_MAX};
    for (int i = gtid; i < k; i += gthreads) b = better(b, Best{sp_mag(AP[pidx(i, k)]), i});
    b = block_best(b, shb);
    double* pvb = pv + (size_t)parity * gridDim.x;
    int* pib = pi + (size_t)parity * gridDim.x;
    if (threadIdx.x == 0) { pvb[blockIdx.x] = b.v; pib[blockIdx.x] = b.i; }
    grid.sync();
    // ---- phase B: pivot choice, identical in every block
    if (threadIdx.x == 0) {
      Best c = {-1.0, INT_MAX};
      for (int q = 0; q < (int)gridDim.x; q++) c = better(c, Best{pvb[q], pib[q]});
      s_col = c;
    }
    __syncthreads();
    parity ^= 1;
    const double colmax = k > 0 ? s_col.v : 0.0;
    const int imax = s_col.i;
    int kp = k, kstep = 1;
    if (fmax(absakk, colmax) == 0.0) {
      // column k is zero: record it and go on (dsptrf: INFO = K, KP = K)
      if (gtid == 0) {
        if (*info == 0) *info = k + 1;
        ipiv[k] = k + 1;
      }
      k -= 1;
      continue;
    }
    if (!(absakk >= alpha * colmax)) {
      // largest off-diagonal magnitude in row/column imax of the leading block
      double rm = 0.0;
      for (int j = imax + 1 + gtid; j <= k; j += gthreads) rm = fmax(rm, sp_mag(AP[pidx(imax, j)]));
      for (int i = gtid; i < imax; i += gthreads) rm = fmax(rm, sp_mag(AP[pidx(i, imax)]));
      rm = block_max(rm, shd);
      if (threadIdx.x == 0) pr[blockIdx.x] = rm;
      const double absimax = sp_mag(AP[pidx(imax, imax)]);
      grid.sync();
      if (threadIdx.x == 0) {
        double r = 0.0;
        for (int q = 0; q < (int)gridDim.x; q++) r = fmax(r, pr[q]);
        s_row = r;
      }
      __syncthreads();
      const double rowmax = s_row;
      if (absakk >= alpha * colmax * (colmax / rowmax)) kp = k;
      else if (absimax >= alpha * rowmax) kp = imax;
      else { kp = imax; kstep = 2; }
    }
    const int kk = k - kstep + 1;
    // ---- phase C: interchange rows and columns kk and kp of the leading block
    if (kp != kk) {
      for (int t = gtid; t < kk; t += gthreads) {
        if (t < kp) sp_swap(AP, pidx(t, kk), pidx(t, kp));
        else if (t > kp) sp_swap(AP, pidx(t, kk), pidx(kp, t));
        else {
          sp_swap(AP, pidx(kk, kk), pidx(kp, kp));
          if (kstep == 2) sp_swap(AP, pidx(k - 1, k), pidx(kp, k));
        }
      }
      grid.sync();
    }
    // ---- phase D: update of the leading block
    if (kstep == 1) {
      r1 = sp_div(one, AP[pidx(k, k)]);
      for (int j = gwarp; j < k; j += gwarps) {
        const T tj = sp_neg(r1) * AP[pidx(j, k)];
        const size_t cj = pidx(0, j), ck = pidx(0, k);
        for (int i = lane; i <= j; i += 32) AP[cj + i] = AP[cj + i] + AP[ck + i] * tj;
      }
      kind = 1;
    } else if (k > 1) {
      d12 = AP[pidx(k - 1, k)];
      d22 = sp_div(AP[pidx(k - 1, k - 1)], d12);
      d11 = sp_div(AP[pidx(k, k)], d12);
      const T t = sp_div(one, d11 * d22 - one);
      d12 = sp_div(t, d12);
      for (int j = gwarp; j < k - 1; j += gwarps) {
        const T a = AP[pidx(j, k - 1)], bb = AP[pidx(j, k)];
        const T wkm1 = d12 * (d11 * a - bb);
        const T wk = d12 * (d22 * bb - a);
        const size_t cj = pidx(0, j), ck = pidx(0, k), ck1 = pidx(0, k - 1);
        for (int i = lane; i <= j; i += 32) AP[cj + i] = AP[cj + i] - AP[ck + i] * wk - AP[ck1 + i] * wkm1;
      }
      kind = 2;
    }
    kc = k;
    if (gtid == 0) {
      if (kstep == 1) ipiv[k] = kp + 1;
      else { ipiv[k] = -(kp + 1); ipiv[k - 1] = -(kp + 1); }
    }
    grid.sync();
    k -= kstep;
  }
  store_multipliers(AP, kind, kc, r1, d11, d22, d12, gtid, gthreads);
}

// dsptrs / zsptrs 'U': one warp per right-hand side (column r of B)
template <typename T>
__global__ void __launch_bounds__(SP_THREADS) sptrs_kernel(const T* AP, int N, const int* ipiv, T* B, long long ldb,
                                                           int nrhs) {
  const int r = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nrhs) return;
  T* b = B + (long long)r * ldb;
  const T one = sp_one<T>();
  // U D X = B, k from N-1 down
  int k = N - 1;
  while (k >= 0) {
    if (ipiv[k] > 0) {
      const int kp = ipiv[k] - 1;
      if (kp != k && lane == 0) { const T t = b[k]; b[k] = b[kp]; b[kp] = t; }
      __syncwarp();
      const T bk = b[k];
      const size_t ck = pidx(0, k);
      for (int i = lane; i < k; i += 32) b[i] = b[i] - AP[ck + i] * bk;
      __syncwarp();
      if (lane == 0) b[k] = sp_div(one, AP[ck + k]) * b[k];
      __syncwarp();
      k -= 1;
    } else {
      const int kp = -ipiv[k] - 1;
      if (kp != k - 1 && lane == 0) { const T t = b[k - 1]; b[k - 1] = b[kp]; b[kp] = t; }
      __syncwarp();
      const T bk = b[k], bk1 = b[k - 1];
      const size_t ck = pidx(0, k), ck1 = pidx(0, k - 1);
      for (int i = lane; i < k - 1; i += 32) {
        T v = b[i] - AP[ck + i] * bk;
        b[i] = v - AP[ck1 + i] * bk1;
      }
      __syncwarp();
      if (lane == 0) {
        const T akm1k = AP[ck + k - 1];
        const T akm1 = sp_div(AP[ck1 + k - 1], akm1k);
        const T ak = sp_div(AP[ck + k], akm1k);
        const T denom = akm1 * ak - one;
        const T bkm1 = sp_div(b[k - 1], akm1k);
        const T bkk = sp_div(b[k], akm1k);
        b[k - 1] = sp_div(ak * bkm1 - bkk, denom);
        b[k] = sp_div(akm1 * bkk - bkm1, denom);
      }
      __syncwarp();
      k -= 2;
    }
  }
  // U^T X = B, k from 0 up
  k = 0;
  while (k < N) {
    const int nb = ipiv[k] > 0 ? 1 : 2;
    for (int c = 0; c < nb; c++) {
      const size_t ck = pidx(0, k + c);
      T acc = sp_zero<T>();
      for (int i = lane; i < k; i += 32) acc = acc + b[i] * AP[ck + i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc = acc + shfl_xor_any(acc, o);
      __syncwarp();
      if (lane == 0) b[k + c] = b[k + c] - acc;
      __syncwarp();
    }
    const int kp = nb == 1 ? ipiv[k] - 1 : -ipiv[k] - 1;
    if (kp != k && lane == 0) { const T t = b[k]; b[k] = b[kp]; b[kp] = t; }
    __syncwarp();
    k += nb;
  }
}

template <typename T>
__global__ void pack_upper(const T* A, long long lda, int n, T* AP) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  for (int j = w; j < n; j += nw)
    for (int i = lane; i <= j; i += 32) AP[pidx(i, j)] = A[i + (long long)j * lda];
}

}  // namespace

// Factor the device packed array dAP (N, dtype F64 or C128) in place; dipiv
// receives LAPACK's 1-based pivot codes; *h_info dsptrf's INFO.
gbem_status sp_factor_device(void* dAP, int N, int dtype, int* dipiv, int* h_info, cudaStream_t s) {
  int dev = 0, nsm = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const void* kern = dtype == GBEM_C128 ? (const void*)sptrf_kernel<cx<double>> : (const void*)sptrf_kernel<double>;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, SP_THREADS, 0);
  if (e != cudaSuccess) return cuda_status(e, "sptrf occupancy");
  // enough warps to give every column of the leading block its own warp,
  // never more blocks than are resident at once (cooperative launch)
  const int want = std::max(1, (int)(((long long)N + SP_THREADS / 32 - 1) / (SP_THREADS / 32)));
  const int G = std::max(1, std::min(nsm * std::max(per, 1), want));
  double *pv = nullptr, *pr = nullptr;
  int *pi = nullptr, *dinfo = nullptr;
  e = cudaMallocAsync((void**)&pv, sizeof(double) * 2 * G, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&pr, sizeof(double) * G, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&pi, sizeof(int) * 2 * G, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dinfo, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dinfo, 0, sizeof(int), s);
  if (e == cudaSuccess) {
    int n = N;
    void* args[] = {&dAP, &n, &dipiv, &dinfo, &pv, &pi, &pr};
    e = cudaLaunchCooperativeKernel(kern, dim3(G), dim3(SP_THREADS), args, 0, s);
    stats_launch(ST_PANEL);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(pv, s); cudaFreeAsync(pr, s); cudaFreeAsync(pi, s); cudaFreeAsync(dinfo, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = e2;
  return e == cudaSuccess ? GBEM_OK : cuda_status(e, "sptrf");
}

gbem_status sp_solve_device(const void* dAP, int N, int dtype, const int* dipiv, int nrhs, void* dB, int ldb,
                            cudaStream_t s) {
  const unsigned grid = (unsigned)((nrhs + SP_THREADS / 32 - 1) / (SP_THREADS / 32));
  if (dtype == GBEM_C128)
    sptrs_kernel<cx<double>><<<grid, SP_THREADS, 0, s>>>((const cx<double>*)dAP, N, dipiv, (cx<double>*)dB, ldb,
                                                         nrhs);
  else
    sptrs_kernel<double><<<grid, SP_THREADS, 0, s>>>((const double*)dAP, N, dipiv, (double*)dB, ldb, nrhs);
  stats_launch(ST_SOLVE);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBEM_OK : cuda_status(e, "sptrs");
}

gbem_status sp_pack_device(const void* dA, int lda, int n, int dtype, void* dAP, cudaStream_t s) {
  const unsigned grid = (unsigned)std::min(4096, (n + 7) / 8);
  if (dtype == GBEM_C128)
    pack_upper<cx<double>><<<grid, 256, 0, s>>>((const cx<double>*)dA, lda, n, (cx<double>*)dAP);
  else
    pack_upper<double><<<grid, 256, 0, s>>>((const double*)dA, lda, n, (double*)dAP);
  stats_launch(ST_OTHER);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBEM_OK : cuda_status(e, "pack");
}

}  // namespace gbem
