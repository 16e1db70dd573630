// lu.cu -- dense complex LU factorisation with partial pivoting, triangular
// solves, and the FP64 residual of iterative refinement (replaces
// HMatrix::LUFactorize / LUSolve, libs/libhmat/LBWrappers.cc:151-236, which
// call LAPACK zgetrf_/zgetrs_).
//
// Right-looking blocked LU, column-major, panel width w:
//   panel_kernel  one cooperative launch per panel: the panel's rows are
//                 spread over the CTAs' shared memory; each column needs one
//                 grid-wide barrier (pivot candidates and the candidate rows
//                 are exchanged through double-buffered global stashes, so
//                 row swaps need no second barrier).  Pivots maximise
//                 |Re|+|Im| in FP64 (LAPACK's IZAMAX); ties go to the lowest row.
//   swap_compose / swap_apply  apply the panel's row interchanges outside the panel.
//   trsm_kernel   U12 = L11^{-1} A12 (unit lower triangle).
//   trailing update A22 -= L21 U12: gemm_simt<T> for FP64, the tensor-core
//                 split-BF16 GEMM (gemm_tc.cu) for the complex-FP32 form.
#include <cooperative_groups.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace cg = cooperative_groups;

namespace gbem {

// tensor-core trailing update (gemm_tc.cu); returns false if unavailable
bool tc_gemm_update(cx<float>* C, long long ldc, const cx<float>* A, long long lda, const cx<float>* B,
                    long long ldb, int m, int n, int k, void* ws, size_t ws_bytes, cudaStream_t s, cudaError_t* err);
size_t tc_gemm_ws_bytes(int m, int n, int k);
int tc_gemm_error(bool reset);

// one CTA's pivot candidate: |Re|+|Im| (FP64) and its global row, written
// and read as one 16-byte record
struct __align__(16) Cand {
  double v;
  int i, pad;
};

template <typename T> struct Stash {
  cx<T>* cand_rows;  // [2][G][w]
  cx<T>* diag_row;   // [2][w]
  Cand* cand;        // [2][G]
};

template <typename T> struct PanelArgs {
  cx<T>* A;
  long long ld;
  int N, c0, w, R;
  int* ipiv;   // 0-based global pivot rows for columns c0..c0+w-1
  int* info;   // first zero pivot (1-based), 0 if none
  Stash<T> st;
};

// row stride of the shared-memory panel: w + 4 elements makes the 4 lanes
// x 8 rows of a warp's elimination step hit distinct banks
__host__ __device__ constexpr int panel_stride(int w) { return w + 4; }

// L2-coherent loads (bypass L1) of data other CTAs wrote before a grid barrier
__device__ __forceinline__ cx<float> ldcg_cx(const cx<float>* p) {
  float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return mk(v.x, v.y);
}
__device__ __forceinline__ cx<double> ldcg_cx(const cx<double>* p) {
  double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return mk(v.x, v.y);
}
__device__ __forceinline__ Cand ldcg_cand(const Cand* p) {
  int4 r = __ldcg(reinterpret_cast<const int4*>(p));
  Cand c;
  c.v = __hiloint2double(r.y, r.x);
  c.i = r.z;
  c.pad = r.w;
  return c;
}

// asynchronous global -> shared copies (8 or 16 bytes), all in flight at once
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)), "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)), "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
template <typename T>
__device__ __forceinline__ void cp_async_cx(cx<T>* sdst, const cx<T>* gsrc) {
  if constexpr (sizeof(T) == 4) cp_async8(sdst, gsrc);
  else cp_async16(sdst, gsrc);
}

__device__ __forceinline__ void better(double v, int i, double& bv, int& bi) {
  if (i < 0) return;
  if (bi < 0 || v > bv || (v == bv && i < bi)) { bv = v; bi = i; }
}

__device__ __forceinline__ void warp_best(double& bv, int& bi) {
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffff, bv, o);
    int oi = __shfl_down_sync(0xffffffff, bi, o);
    better(ov, oi, bv, bi);
  }
}

// Per column: the elimination of column jj is fused with the local pivot
// search of column jj+1; warp 0 publishes the CTA's candidate record and its
// row, warp 1 the diagonal row; one grid barrier; warp 0 reads all records
// (one 16-byte load per lane and CTA slot, issued together), picks the global
// winner and broadcasts it through shared memory.  The CTA's rows are spread
// over 4 adjacent lanes per row during elimination.
template <typename T>
__global__ void __launch_bounds__(512) panel_kernel(PanelArgs<T> a) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = a.w, wp = panel_stride(a.w);
  cx<T>* rows = reinterpret_cast<cx<T>*>(smem_raw);  // [R][wp]
  cx<T>* u = rows + (size_t)a.R * wp;                 // pivot row [w]
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  __shared__ double s_gv;
  __shared__ int s_p, s_wc;
  const int G = gridDim.x, c = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  const int m0 = a.c0 + c * a.R;
  const int nr = max(0, min(a.R, a.N - m0));
  for (int q = tid; q < nr * w; q += nt) {
    int r = q % nr, k = q / nr;
    rows[r * wp + k] = a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld];
  }
  __syncthreads();
  {  // candidates of column 0
    double bv = -1.0;
    int bi = -1;
    for (int r = tid; r < nr; r += nt) {
      cx<T> z = rows[r * wp];
      better(fabs((double)z.re) + fabs((double)z.im), m0 + r, bv, bi);
    }
    warp_best(bv, bi);
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
  }
  __syncthreads();
  for (int jj = 0; jj < w; jj++) {
    const int d = a.c0 + jj, buf = jj & 1;
    if (warp == 0) {
      double bv = lane < nw ? red_v[lane] : -1.0;
      int bi = lane < nw ? red_i[lane] : -1;
      warp_best(bv, bi);
      bv = __shfl_sync(0xffffffff, bv, 0);
      bi = __shfl_sync(0xffffffff, bi, 0);
      if (lane == 0) {
        Cand cd;
        cd.v = bv; cd.i = bi; cd.pad = 0;
        a.st.cand[buf * G + c] = cd;
      }
      if (bi >= 0)
        for (int k = lane; k < w; k += 32) a.st.cand_rows[((size_t)buf * G + c) * w + k] = rows[(bi - m0) * wp + k];
      __threadfence();
    } else if (warp == 1 && d >= m0 && d < m0 + nr) {
      for (int k = lane; k < w; k += 32) a.st.diag_row[(size_t)buf * w + k] = rows[(d - m0) * wp + k];
      __threadfence();
    }
    grid.sync();
    if (warp == 0) {
      // global winner (ties: lowest row, like IZAMAX); the record loads are
      // independent of one another, so they are all in flight at once
      constexpr int MAXT = 8;  // G <= 256
      Cand rec[MAXT];
#pragma unroll
      for (int t = 0; t < MAXT; t++) {
        const int q = lane + 32 * t;
        if (q < G) rec[t] = ldcg_cand(&a.st.cand[buf * G + q]);
        else { rec[t].v = -1.0; rec[t].i = -1; rec[t].pad = 0; }
      }
      double gv = -1.0;
      int gi = -1, gc = -1;
#pragma unroll
      for (int t = 0; t < MAXT; t++) {
        const int i = rec[t].i;
        const double v = rec[t].v;
        if (i >= 0 && (gi < 0 || v > gv || (v == gv && i < gi))) { gv = v; gi = i; gc = lane + 32 * t; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffff, gv, o);
        int oi = __shfl_down_sync(0xffffffff, gi, o);
        int oc = __shfl_down_sync(0xffffffff, gc, o);
        if (oi >= 0 && (gi < 0 || ov > gv || (ov == gv && oi < gi))) { gv = ov; gi = oi; gc = oc; }
      }
      if (lane == 0) {
        // a missing candidate cannot happen (row d is one); it would read as a zero pivot at d
        if (gi < 0) { gi = d; gc = min(G - 1, (d - a.c0) / a.R); gv = 0.0; }
        s_gv = gv; s_p = gi; s_wc = gc;
        if (c == 0) {
          a.ipiv[d] = gi;
          if (gv == 0.0 && *a.info == 0) *a.info = d + 1;
        }
      }
    }
    __syncthreads();
    const int p = s_p, wc = s_wc;
    const cx<T>* win = a.st.cand_rows + ((size_t)buf * G + wc) * w;
    for (int k = tid; k < w; k += nt) {
      cx<T> x = ldcg_cx(win + k);
      u[k] = x;
      if (d >= m0 && d < m0 + nr) rows[(d - m0) * wp + k] = x;
    }
    if (p != d && p >= m0 && p < m0 + nr)
      for (int k = tid; k < w; k += nt) rows[(p - m0) * wp + k] = ldcg_cx(a.st.diag_row + (size_t)buf * w + k);
    __syncthreads();
    // eliminate column jj (4 adjacent lanes per row) and search column jj+1
    const cx<T> piv = u[jj];
    const T pn = piv.re * piv.re + piv.im * piv.im;
    const cx<T> inv = pn != (T)0 ? mk(piv.re / pn, -piv.im / pn) : mk((T)0, (T)0);
    const int rs = max(0, d + 1 - m0);
    const int cgi = tid & 3, RT = nt >> 2;
    double bv = -1.0;
    int bi = -1;
    for (int rb = rs; rb < nr; rb += RT) {
      const int r = rb + (tid >> 2);
      const bool valid = r < nr;
      cx<T> l = mk((T)0, (T)0);
      if (valid && pn != (T)0) l = rows[r * wp + jj] * inv;
      __syncwarp();
      if (valid) {
        if (pn != (T)0) {
          if (cgi == 0) rows[r * wp + jj] = l;
          for (int k = jj + 1 + cgi; k < w; k += 4) rows[r * wp + k] = rows[r * wp + k] - l * u[k];
        }
        if (cgi == 0 && jj + 1 < w) {
          cx<T> z = rows[r * wp + jj + 1];
          better(fabs((double)z.re) + fabs((double)z.im), m0 + r, bv, bi);
        }
      }
    }
    warp_best(bv, bi);
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
  }
  for (int q = tid; q < nr * w; q += nt) {
    int r = q % nr, k = q / nr;
    a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld] = rows[r * wp + k];
  }
}

// ---------------------------------------------------------------------------
// Leaf of the recursive panel factorisation (complex FP32): columns
// [c0, c0+w) (w <= LEAF_W) of rows [c0, N), held by the CTAs of ONE thread-block
// cluster (rank r owns rows [c0 + r*Rr, c0 + (r+1)*Rr)).  Partial pivoting with
// LAPACK's |Re|+|Im| measure (FP64), ties to the lowest row; per column one
// cluster barrier, with the candidate records, candidate rows and the
// diagonal row exchanged through distributed shared memory.
// ---------------------------------------------------------------------------
constexpr int LEAF_W = 16;
constexpr int LEAF_STRIDE = LEAF_W + 1;  // odd: thread-per-row access is conflict-free

struct LeafArgs {
  cx<float>* A;
  long long ld;
  int N, c0, w, Rr;
  int pc0, pc1;  // the enclosing panel's columns: the leaf's interchanges are applied to all of them
  int* ipiv;     // 0-based global pivot rows
  int* info;
  // register leaves only: first apply the 16-column leaf just left of this
  // one, U12 = L11^-1 A12 (rows c0-16 .. c0-1, stored) and A22 -= L21 U12
  int fuse;
};

__global__ void __launch_bounds__(512) leaf_kernel(LeafArgs a) {
  pdl_wait();
  pdl_trigger();
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<float>* rows = reinterpret_cast<cx<float>*>(smem_raw);  // [Rr][LEAF_STRIDE]
  __shared__ Cand pub[2];
  __shared__ cx<float> prow[2][LEAF_W];
  __shared__ cx<float> drow[2][LEAF_W];
  __shared__ cx<float> u[LEAF_W];
  __shared__ double red_v[16];
  __shared__ int red_i[16];
  __shared__ int s_p, s_own;
  const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  const int w = a.w;
  const int m0 = a.c0 + rank * a.Rr;
  const int nr = max(0, min(a.Rr, a.N - m0));
  for (int q = tid; q < nr * w; q += nt) {
    const int r = q % nr, k = q / nr;
    cp_async8(&rows[r * LEAF_STRIDE + k], &a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld]);
  }
  cp_async_wait_all();
  __syncthreads();
  // this CTA's share of the panel's other columns, whose rows it interchanges
  // one pivot behind (the loads of pivot jj are in flight during column jj+1)
  int scol = -1;
  {
    int cnt = 0;
    for (int col = a.pc0 + rank; col < a.pc1; col += CL) {
      if (col >= a.c0 && col < a.c0 + w) continue;
      if (cnt == tid) scol = col;
      cnt++;
    }
  }
  bool pend = false;
  int pd = 0, pp = 0;
  cx<float> xd = mk(0.0f, 0.0f), xp = xd;
  {
    double bv = -1.0;
    int bi = -1;
    for (int r = tid; r < nr; r += nt) {
      const cx<float> z = rows[r * LEAF_STRIDE];
      better(fabs((double)z.re) + fabs((double)z.im), m0 + r, bv, bi);
    }
    warp_best(bv, bi);
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
  }
  __syncthreads();
  for (int jj = 0; jj < w; jj++) {
    const int d = a.c0 + jj, buf = jj & 1;
    if (warp == 0) {
      double bv = lane < nw ? red_v[lane] : -1.0;
      int bi = lane < nw ? red_i[lane] : -1;
      warp_best(bv, bi);
      bv = __shfl_sync(0xffffffff, bv, 0);
      bi = __shfl_sync(0xffffffff, bi, 0);
      if (lane == 0) { pub[buf].v = bv; pub[buf].i = bi; pub[buf].pad = 0; }
      if (bi >= 0 && lane < w) prow[buf][lane] = rows[(bi - m0) * LEAF_STRIDE + lane];
    } else if (warp == 1 && d >= m0 && d < m0 + nr && lane < w) {
      drow[buf][lane] = rows[(d - m0) * LEAF_STRIDE + lane];
    }
    cl.sync();
    if (warp == 0) {
      double gv = -1.0;
      int gi = -1, gc = -1;
      if (lane < CL) {
        const Cand x = *cl.map_shared_rank(&pub[buf], lane);
        gv = x.v; gi = x.i; gc = lane;
      }
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffff, gv, o);
        int oi = __shfl_down_sync(0xffffffff, gi, o);
        int oc = __shfl_down_sync(0xffffffff, gc, o);
        if (oi >= 0 && (gi < 0 || ov > gv || (ov == gv && oi < gi))) { gv = ov; gi = oi; gc = oc; }
      }
      if (lane == 0) {
        // a missing candidate cannot happen (row d is one); it would read as a zero pivot at d
        if (gi < 0) { gi = d; gc = (d - a.c0) / a.Rr; gv = 0.0; }
        s_p = gi; s_own = gc;
        if (rank == 0) {
          a.ipiv[d] = gi;
          if (gv == 0.0 && *a.info == 0) *a.info = d + 1;
        }
      }
    }
    __syncthreads();
    const int p = s_p, own = s_own;
    if (scol >= 0) {
      cx<float>* colp = a.A + (long long)scol * a.ld;
      if (pend) { colp[pp] = xd; colp[pd] = xp; pend = false; }
      if (p != d && p >= 0) { xd = colp[d]; xp = colp[p]; pd = d; pp = p; pend = true; }
    }
    if (tid < w) {
      const cx<float> x = cl.map_shared_rank(&prow[buf][0], own)[tid];
      u[tid] = x;
      if (d >= m0 && d < m0 + nr) rows[(d - m0) * LEAF_STRIDE + tid] = x;
      if (p != d && p >= m0 && p < m0 + nr)
        rows[(p - m0) * LEAF_STRIDE + tid] = cl.map_shared_rank(&drow[buf][0], (d - a.c0) / a.Rr)[tid];
    }
    __syncthreads();
    // eliminate column jj (one thread per row) and search column jj+1
    const cx<float> piv = u[jj];
    const float pn = piv.re * piv.re + piv.im * piv.im;
    const cx<float> inv = pn != 0.0f ? mk(piv.re / pn, -piv.im / pn) : mk(0.0f, 0.0f);
    double bv = -1.0;
    int bi = -1;
    for (int r = max(0, d + 1 - m0) + tid; r < nr; r += nt) {
      cx<float>* row = rows + r * LEAF_STRIDE;
      if (pn != 0.0f) {
        const cx<float> l = row[jj] * inv;
        row[jj] = l;
        for (int k = jj + 1; k < w; k++) row[k] = row[k] - l * u[k];
      }
      if (jj + 1 < w) {
        const cx<float> z = row[jj + 1];
        better(fabs((double)z.re) + fabs((double)z.im), m0 + r, bv, bi);
      }
    }
    warp_best(bv, bi);
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
  }
  if (pend) {
    cx<float>* colp = a.A + (long long)scol * a.ld;
    colp[pp] = xd;
    colp[pd] = xp;
  }
  // no CTA leaves while another may still read its shared memory
  cl.sync();
  for (int q = tid; q < nr * w; q += nt) {
    const int r = q % nr, k = q / nr;
    a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld] = rows[r * LEAF_STRIDE + k];
  }
}

// Register-resident leaf (same contract as leaf_kernel): each thread holds RT
// rows of the leaf (r = tid + t * 512) in registers, so elimination is pure
// register arithmetic.  Pivot search uses LAPACK's complex-FP32 measure
// |Re|+|Im| in FP32 (ICAMAX), first maximum; warp candidates come from
// redux.sync max/min, the CTA candidate from warp 0, the cluster winner from
// the CTAs' records in distributed shared memory.  Three barriers per column
// (one of them the cluster barrier).
__device__ __forceinline__ void warp_cand(unsigned vb, int row, unsigned& wvb, int& wrow) {
  const unsigned mx = __reduce_max_sync(0xffffffffu, vb);
  const int cand = (vb == mx && row >= 0) ? row : 0x7fffffff;
  wvb = mx;
  wrow = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
}

template <int RT, int NT>
__global__ void __launch_bounds__(NT, 1) leaf_kernel_reg(LeafArgs a) {
  pdl_wait();
  pdl_trigger();
  cg::cluster_group cl = cg::this_cluster();
  __shared__ Cand pub[2];
  __shared__ __align__(16) cx<float> prow[2][LEAF_W];
  __shared__ __align__(16) cx<float> drow[2][LEAF_W];
  constexpr int NW = NT / 32;
  __shared__ __align__(16) cx<float> wrow[NW][LEAF_W];
  __shared__ unsigned w_vb[NW];
  __shared__ int w_row[NW];
  __shared__ __align__(16) cx<float> allrows[16][LEAF_W];  // every CTA's candidate row
  __shared__ __align__(16) cx<float> dcopy[LEAF_W];        // the diagonal row before the interchange
  __shared__ int s_p, s_own;
  const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int w = a.w;
  const int m0 = a.c0 + rank * a.Rr;
  const int nr = max(0, min(a.Rr, a.N - m0));
  cx<float> R[RT][LEAF_W];
#pragma unroll
  for (int t = 0; t < RT; t++) {
    const int r = tid + t * NT;
#pragma unroll
    for (int k = 0; k < LEAF_W; k++)
      R[t][k] = (r < nr && k < w) ? a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld] : mk(0.0f, 0.0f);
  }
  // the panel's other columns whose rows this CTA interchanges, one pivot behind
  int scol = -1;
  {
    int cnt = 0;
    for (int col = a.pc0 + rank; col < a.pc1; col += CL) {
      if (col >= a.c0 && col < a.c0 + w) continue;
      if (cnt == tid) scol = col;
      cnt++;
    }
  }
  bool pend = false;
  int pd = 0, pp = 0;
  cx<float> xd = mk(0.0f, 0.0f), xp = xd;
  __shared__ __align__(16) cx<float> u12[LEAF_W][LEAF_W + 1];
  if (a.fuse) {
    // the previous leaf's block row: U12 = L11^-1 A12 (L11 unit lower), every
    // CTA for itself, then A22 -= L21 U12 on this CTA's rows
    __shared__ __align__(16) cx<float> l11[LEAF_W][LEAF_W + 1];
    const int lc = a.c0 - LEAF_W;
    for (int q = tid; q < LEAF_W * LEAF_W; q += NT) {
      const int i = q % LEAF_W, j = q / LEAF_W;
      l11[i][j] = a.A[(lc + i) + (long long)(lc + j) * a.ld];
      u12[i][j] = j < w ? a.A[(lc + i) + (long long)(a.c0 + j) * a.ld] : mk(0.0f, 0.0f);
    }
    __syncthreads();
    if (tid < w) {
      for (int i = 1; i < LEAF_W; i++) {
        cx<float> acc = u12[i][tid];
        for (int kk = 0; kk < i; kk++) acc = acc - l11[i][kk] * u12[kk][tid];
        u12[i][tid] = acc;
      }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < RT; t++) {
      const int r = tid + t * NT;
      if (r < nr) {
        cx<float> l[LEAF_W];
#pragma unroll
        for (int i = 0; i < LEAF_W; i++) l[i] = a.A[(m0 + r) + (long long)(lc + i) * a.ld];
#pragma unroll
        for (int kk = 0; kk < LEAF_W; kk++) {
          cx<float> acc = R[t][kk];
#pragma unroll
          for (int i = 0; i < LEAF_W; i++) acc = acc - l[i] * u12[i][kk];
          R[t][kk] = acc;
        }
      }
    }
  }
  // candidates of column 0
  unsigned cvb = 0u;
  int crow = -1;
#pragma unroll
  for (int t = 0; t < RT; t++) {
    const int r = tid + t * NT;
    if (r < nr) {
      const unsigned vb = __float_as_uint(fabsf(R[t][0].re) + fabsf(R[t][0].im));
      if (crow < 0 || vb > cvb) { cvb = vb; crow = m0 + r; }
    }
  }
#pragma unroll
  for (int jj = 0; jj < LEAF_W; jj++) {
    if (jj >= w) break;
    const int d = a.c0 + jj, buf = jj & 1;
    // warp candidate; its owner lane stages the row; the owner of row d stages it too
    {
      unsigned wvb;
      int wr;
      warp_cand(cvb, crow, wvb, wr);
      if (lane == 0) { w_vb[warp] = wvb; w_row[warp] = wr; }
#pragma unroll
      for (int t = 0; t < RT; t++) {
        const int g = m0 + tid + t * NT;
        if (tid + t * NT < nr) {
          if (g == wr)
#pragma unroll
            for (int k = 0; k < LEAF_W; k++) wrow[warp][k] = R[t][k];
          if (g == d)
#pragma unroll
            for (int k = 0; k < LEAF_W; k++) drow[buf][k] = R[t][k];
        }
      }
    }
    __syncthreads();
    if (warp == 0) {
      const unsigned vb = lane < NW ? w_vb[lane] : 0u;
      const int rw = lane < NW ? w_row[lane] : 0x7fffffff;
      const unsigned mx = __reduce_max_sync(0xffffffffu, rw != 0x7fffffff ? vb : 0u);
      const int cand = (rw != 0x7fffffff && vb == mx) ? rw : 0x7fffffff;
      const int best = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
      const unsigned who = __ballot_sync(0xffffffffu, rw == best && best != 0x7fffffff);
      const int bw = who ? __ffs(who) - 1 : 0;
      if (lane == 0) {
        pub[buf].v = best != 0x7fffffff ? (double)__uint_as_float(mx) : -1.0;
        pub[buf].i = best != 0x7fffffff ? best : -1;
        pub[buf].pad = 0;
      }
      if (lane < LEAF_W && best != 0x7fffffff) prow[buf][lane] = wrow[bw][lane];
    }
    cl.sync();
    // one round trip through distributed shared memory: every CTA's record and
    // candidate row, and the diagonal row, read in parallel
    if (tid < 16 * LEAF_W) {
      const int rk = tid / LEAF_W, k = tid % LEAF_W;
      if (rk < CL && k < w) allrows[rk][k] = cl.map_shared_rank(&prow[buf][0], rk)[k];
    } else if (tid < 17 * LEAF_W) {
      const int k = tid - 16 * LEAF_W;
      if (k < w) dcopy[k] = cl.map_shared_rank(&drow[buf][0], (d - a.c0) / a.Rr)[k];
    } else if (warp == 9) {
      unsigned vb = 0u;
      int ri = 0x7fffffff;
      if (lane < CL) {
        const Cand x = *cl.map_shared_rank(&pub[buf], lane);
        if (x.i >= 0) { vb = __float_as_uint((float)x.v); ri = x.i; }
      }
      const unsigned mx = __reduce_max_sync(0xffffffffu, vb);
      const int cand = (ri != 0x7fffffff && vb == mx) ? ri : 0x7fffffff;
      const int best = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
      const unsigned who = __ballot_sync(0xffffffffu, lane < CL && ri == best);
      const int own = who ? __ffs(who) - 1 : 0;
      if (lane == 0) {
        // no candidate anywhere cannot happen (row d itself is one); treat it
        // as a zero pivot at d so no index is ever out of range
        s_p = best != 0x7fffffff ? best : d;
        s_own = own;
        if (rank == 0) {
          a.ipiv[d] = best != 0x7fffffff ? best : d;
          if ((mx == 0u || best == 0x7fffffff) && *a.info == 0) *a.info = d + 1;
        }
      }
    }
    __syncthreads();
    const cx<float>* u = allrows[s_own];  // the pivot row
    const int p = s_p;
    if (scol >= 0) {
      cx<float>* colp = a.A + (long long)scol * a.ld;
      if (pend) { colp[pp] = xd; colp[pd] = xp; pend = false; }
      if (p != d && p > d && p < a.N) { xd = colp[d]; xp = colp[p]; pd = d; pp = p; pend = true; }
    }
    // interchange rows d and p in registers, eliminate column jj, search jj+1
    const cx<float> piv = u[jj];
    const float pn = piv.re * piv.re + piv.im * piv.im;
    const cx<float> inv = pn != 0.0f ? mk(piv.re / pn, -piv.im / pn) : mk(0.0f, 0.0f);
    cvb = 0u;
    crow = -1;
#pragma unroll
    for (int t = 0; t < RT; t++) {
      const int r = tid + t * NT, g = m0 + r;
      if (r < nr) {
        if (g == d) {
#pragma unroll
          for (int k = 0; k < LEAF_W; k++) R[t][k] = u[k];
        } else if (g == p) {
#pragma unroll
          for (int k = 0; k < LEAF_W; k++) R[t][k] = dcopy[k];
        }
        if (g > d) {
          if (pn != 0.0f) {
            const cx<float> l = R[t][jj] * inv;
            R[t][jj] = l;
#pragma unroll
            for (int k = jj + 1; k < LEAF_W; k++) R[t][k] = R[t][k] - l * u[k];
          }
          if (jj + 1 < LEAF_W) {
            const unsigned vb = __float_as_uint(fabsf(R[t][jj + 1].re) + fabsf(R[t][jj + 1].im));
            if (crow < 0 || vb > cvb) { cvb = vb; crow = g; }
          }
        }
      }
    }
  }
  if (pend) {
    cx<float>* colp = a.A + (long long)scol * a.ld;
    colp[pp] = xd;
    colp[pd] = xp;
  }
  // no CTA leaves while another may still read its shared memory (and every
  // CTA has read A12 before it is overwritten with U12)
  cl.sync();
#pragma unroll
  for (int t = 0; t < RT; t++) {
    const int r = tid + t * NT;
    if (r < nr)
#pragma unroll
      for (int k = 0; k < LEAF_W; k++)
        if (k < w) a.A[(m0 + r) + (long long)(a.c0 + k) * a.ld] = R[t][k];
  }
  if (a.fuse && rank == 0)
    for (int q = tid; q < LEAF_W * w; q += NT) {
      const int i = q % LEAF_W, j = q / LEAF_W;
      a.A[(a.c0 - LEAF_W + i) + (long long)(a.c0 + j) * a.ld] = u12[i][j];
    }
}

// Row interchanges outside a panel, in two steps.  swap_compose (one CTA)
// folds the panel's interchanges (rows [r0, r1) with ipiv, LAPACK order) into
// the list of rows whose content moves: mv[2e] = destination row, mv[2e+1] =
// the row it takes its content from; rows beyond the panel are tracked in a
// shared-memory hash table (pivots are always at or below their row).  Then
// swap_apply moves each column's rows with one gather per listed row, all
// loads of a column before its stores -- no chain of dependent swaps, and
// nothing to do for rows that pivot on the diagonal.
constexpr int SWAP_HASH = 1024;  // >= 2 x the widest panel (256)

__global__ void __launch_bounds__(256) swap_compose(const int* ipiv, int r0, int r1, int* mv, int* mv_n) {
  pdl_wait();
  pdl_trigger();
  __shared__ int psrc[256];
  __shared__ int hkey[SWAP_HASH], hval[SWAP_HASH];
  __shared__ int cnt;
  const int w = r1 - r0;
  for (int i = threadIdx.x; i < w; i += blockDim.x) psrc[i] = r0 + i;
  for (int i = threadIdx.x; i < SWAP_HASH; i += blockDim.x) hkey[i] = -1;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = r0; i < r1; i++) {
      const int p = ipiv[i];
      if (p == i) continue;
      const int si = psrc[i - r0];
      if (p < r1) {
        psrc[i - r0] = psrc[p - r0];
        psrc[p - r0] = si;
      } else {
        unsigned h = ((unsigned)p * 2654435761u) >> 22;  // 10 bits
        while (hkey[h] != -1 && hkey[h] != p) h = (h + 1) & (SWAP_HASH - 1);
        const int sp = hkey[h] == p ? hval[h] : p;
        hkey[h] = p;
        hval[h] = si;
        psrc[i - r0] = sp;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < w; i += blockDim.x)
    if (psrc[i] != r0 + i) {
      const int e = atomicAdd(&cnt, 1);
      mv[2 * e] = r0 + i; mv[2 * e + 1] = psrc[i];
    }
  for (int i = threadIdx.x; i < SWAP_HASH; i += blockDim.x)
    if (hkey[i] != -1 && hval[i] != hkey[i]) {
      const int e = atomicAdd(&cnt, 1);
      mv[2 * e] = hkey[i]; mv[2 * e + 1] = hval[i];
    }
  __syncthreads();
  if (threadIdx.x == 0) *mv_n = cnt;
}

// one warp per column of [cb, ce) outside [skip0, skip1); at most 2 x 256 moved rows
template <typename T>
__global__ void __launch_bounds__(256) swap_apply(cx<T>* A, long long ld, const int* mv, const int* mv_n, int cb, int ce,
                                                  int skip0, int skip1) {
  pdl_wait();
  pdl_trigger();
  const int j = cb + (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (j >= ce || (j >= skip0 && j < skip1)) return;  // whole warps leave together
  const int n = *mv_n;
  cx<T>* col = A + (long long)j * ld;
  cx<T> v[16];
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const int e = lane + 32 * q;
    if (e < n) v[q] = col[mv[2 * e + 1]];
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const int e = lane + 32 * q;
    if (e < n) col[mv[2 * e]] = v[q];
  }
}

// U12 = L11^{-1} A12: rows [c0, c0+w), columns [cb, ce), 32 columns per CTA.
// L11 is walked in 32 x 32 tiles (each diagonal tile, then the tiles below it)
// through two shared-memory buffers: the next tile's cp.async copy is in
// flight while the current one is used.  A diagonal tile is a short
// sequential solve, a tile below it a small GEMM update.  Used where L11 is
// not made of whole 32-row blocks (trsm_blocked otherwise).
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

template <typename T>
__global__ void __launch_bounds__(256) trsm_kernel(cx<T>* A, long long ld, int c0, int w, int cb, int ce) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* B = reinterpret_cast<cx<T>*>(smem_raw);  // [w][33]
  __shared__ __align__(16) cx<T> Lt[2][32][33];    // cp.async targets: element-aligned
  const int j0 = cb + blockIdx.x * 32;
  const int nc = min(32, ce - j0);
  const int tid = threadIdx.x;
  auto issue = [&](int buf, int kb, int ib) {
    const int kn = min(32, w - kb), in = min(32, w - ib);
    for (int q = tid; q < in * kn; q += blockDim.x) {
      const int i = q % in, k = q / in;
      cp_async_cx(&Lt[buf][i][k], &A[(c0 + ib + i) + (long long)(c0 + kb + k) * ld]);
    }
  };
  for (int q = tid; q < w * nc; q += blockDim.x) {
    const int i = q % w, j = q / w;
    cp_async_cx(&B[i * 33 + j], &A[(c0 + i) + (long long)(j0 + j) * ld]);
  }
  issue(0, 0, 0);
  cp_async_commit();
  int buf = 0;
  for (int kb = 0; kb < w; kb += 32) {
    const int kn = min(32, w - kb);
    for (int ib = kb; ib < w; ib += 32) {
      int nkb = kb, nib = ib + 32;
      if (nib >= w) { nkb = kb + 32; nib = nkb; }
      if (nkb < w) issue(buf ^ 1, nkb, nib);
      cp_async_commit();
      cp_async_wait_1();
      __syncthreads();
      if (ib == kb) {
        // diagonal tile: unit lower solve, columns in parallel
        for (int k = 0; k < kn - 1; k++) {
          for (int q = tid; q < (kn - k - 1) * nc; q += blockDim.x) {
            const int i = k + 1 + q % (kn - k - 1), j = q / (kn - k - 1);
            B[(kb + i) * 33 + j] = B[(kb + i) * 33 + j] - Lt[buf][i][k] * B[(kb + k) * 33 + j];
          }
          __syncthreads();
        }
      } else {
        // tile below: B[ib] -= L[ib, kb] * B[kb]
        const int in = min(32, w - ib);
        for (int q = tid; q < in * nc; q += blockDim.x) {
          const int i = q % in, j = q / in;
          cx<T> acc = mk((T)0, (T)0);
          for (int k = 0; k < kn; k++) acc = acc + Lt[buf][i][k] * B[(kb + k) * 33 + j];
          B[(ib + i) * 33 + j] = B[(ib + i) * 33 + j] - acc;
        }
      }
      __syncthreads();
      buf ^= 1;
    }
  }
  for (int q = tid; q < w * nc; q += blockDim.x) {
    const int i = q % w, j = q / w;
    A[(c0 + i) + (long long)(j0 + j) * ld] = B[i * 33 + j];
  }
}

// U12 = L11^{-1} A12 with the inverted diagonal blocks (w a multiple of 32,
// c0 of 32): the unit-lower inverses of the 32 x 32 diagonal blocks of L live
// in dinv (1024 elements per block, slot row/32, column-major); a block whose
// bit is set in make is inverted here first (31 barriers, every CTA; CTA 0
// stores it), every later solve reads it.  32 columns per CTA, one 32-row
// block step at a time: x_b = D_b^-1 y_b, then every row below the block at
// once, y -= L(rows below, b) x_b, from a column block of L staged in shared
// memory.  Thread (lane j, warp g) owns column j: rows 4g..4g+3 of x_b and
// rows g, g+8, ... below, with the column's 32 values of x_b in registers,
// so the only shared-memory operand per complex MAC is an L element that
// the whole warp reads at once (a broadcast).  Three barriers per block step.
template <typename T>
__global__ void __launch_bounds__(256) trsm_blocked(cx<T>* A, long long ld, int c0, int w, int cb, int ce, cx<T>* dinv,
                                                    unsigned make) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* B = reinterpret_cast<cx<T>*>(smem_raw);  // [w][33]
  cx<T>* Lc = B + w * 33;                          // [w][33]: the column block of L at and below the diagonal
  cx<T>* Dt = Lc + w * 33;                         // [32][33]
  const int j0 = cb + blockIdx.x * 32;
  const int nc = min(32, ce - j0);
  const int tid = threadIdx.x, lane = tid & 31, g = tid >> 5;
  for (int q = tid; q < w * 32; q += blockDim.x) {
    const int i = q % w, j = q / w;
    if (j < nc) cp_async_cx(&B[i * 33 + j], &A[(c0 + i) + (long long)(j0 + j) * ld]);
  }
  cp_async_commit();
  for (int kb = 0; kb < w; kb += 32) {
    // L(kb.., kb..kb+32): the diagonal tile and everything below it
    const int R = w - kb;
    for (int q = tid; q < R * 32; q += blockDim.x) {
      const int i = q % R, k = q / R;
      cp_async_cx(&Lc[i * 33 + k], &A[(c0 + kb + i) + (long long)(c0 + kb + k) * ld]);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    cx<T>* slot = dinv + (size_t)((c0 + kb) / 32) * 1024;
    if ((make >> (kb / 32)) & 1u) {
      for (int q = tid; q < 1024; q += blockDim.x) Dt[(q % 32) * 33 + q / 32] = mk((T)(q % 32 == q / 32), (T)0);
      __syncthreads();
      for (int k = 0; k < 31; k++) {
        for (int q = tid; q < (31 - k) * (k + 1); q += blockDim.x) {
          const int i = k + 1 + q % (31 - k), jj = q / (31 - k);
          Dt[i * 33 + jj] = Dt[i * 33 + jj] - Lc[i * 33 + k] * Dt[k * 33 + jj];
        }
        __syncthreads();
      }
      if (blockIdx.x == 0)
        for (int q = tid; q < 1024; q += blockDim.x) slot[q] = Dt[(q % 32) * 33 + q / 32];
    } else {
      for (int q = tid; q < 1024; q += blockDim.x) Dt[(q % 32) * 33 + q / 32] = slot[q];
      __syncthreads();
    }
    // x_b = D^-1 y_b: rows 4g..4g+3 of column lane
    cx<T> x[4];
#pragma unroll
    for (int t = 0; t < 4; t++) x[t] = mk((T)0, (T)0);
    for (int k = 0; k < 4 * g + 4; k++) {
      const cx<T> y = B[(kb + k) * 33 + lane];
#pragma unroll
      for (int t = 0; t < 4; t++)
        if (k <= 4 * g + t) x[t] = x[t] + Dt[(4 * g + t) * 33 + k] * y;
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; t++) B[(kb + 4 * g + t) * 33 + lane] = x[t];
    __syncthreads();
    // rows below the block: y_i -= sum_k L(i, k) x_k, with the column's x_b in
    // registers and L(i, k) a broadcast over the warp
    cx<T> xb[32];
#pragma unroll
    for (int k = 0; k < 32; k++) xb[k] = B[(kb + k) * 33 + lane];
    for (int i = 32 + g; i < R; i += 8) {
      cx<T> acc = mk((T)0, (T)0);
#pragma unroll
      for (int k = 0; k < 32; k++) acc = acc + Lc[i * 33 + k] * xb[k];
      B[(kb + i) * 33 + lane] = B[(kb + i) * 33 + lane] - acc;
    }
    __syncthreads();
  }
  for (int q = tid; q < w * nc; q += blockDim.x) {
    const int i = q % w, j = q / w;
    A[(c0 + i) + (long long)(j0 + j) * ld] = B[i * 33 + j];
  }
}

// unit-lower inverses of the 32 x 32 diagonal blocks of columns [c0, c0+w)
// (w a multiple of 32), one CTA per block, into dinv's slots (see trsm_blocked)
template <typename T>
__global__ void __launch_bounds__(256) tri_inv_blocks(const cx<T>* A, long long ld, int c0, cx<T>* dinv) {
  pdl_wait();
  pdl_trigger();
  __shared__ cx<T> L[32][33], X[32][33];
  const int r0 = c0 + 32 * blockIdx.x, tid = threadIdx.x;
  for (int q = tid; q < 1024; q += blockDim.x) {
    const int i = q % 32, k = q / 32;
    L[i][k] = A[(r0 + i) + (long long)(r0 + k) * ld];
    X[i][k] = mk((T)(i == k), (T)0);
  }
  __syncthreads();
  for (int k = 0; k < 31; k++) {
    for (int q = tid; q < (31 - k) * (k + 1); q += blockDim.x) {
      const int i = k + 1 + q % (31 - k), j = q / (31 - k);
      X[i][j] = X[i][j] - L[i][k] * X[k][j];
    }
    __syncthreads();
  }
  cx<T>* slot = dinv + (size_t)(r0 / 32) * 1024;
  for (int q = tid; q < 1024; q += blockDim.x) slot[q] = X[q % 32][q / 32];
}

// C -= A B (complex, column-major), 64x64 tiles, 4x4 outputs per thread
template <typename T>
__global__ void __launch_bounds__(256) gemm_simt(cx<T>* C, long long ldc, const cx<T>* A, long long lda,
                                                 const cx<T>* B, long long ldb, int m, int n, int K) {
  pdl_wait();
  pdl_trigger();
  __shared__ cx<T> As[16][64 + 1];
  __shared__ cx<T> Bs[16][64 + 1];
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  cx<T> acc[4][4];
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) acc[a][b] = mk((T)0, (T)0);
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int q = threadIdx.x; q < 16 * 64; q += 256) {
      int ii = q % 64, kk = q / 64;
      int gi = i0 + ii, gk = k0 + kk;
      As[kk][ii] = (gi < m && gk < K) ? A[gi + (long long)gk * lda] : mk((T)0, (T)0);
      int jj = q / 16, kb = q % 16;
      int gj = j0 + jj, gkb = k0 + kb;
      Bs[kb][jj] = (gj < n && gkb < K) ? B[gkb + (long long)gj * ldb] : mk((T)0, (T)0);
    }
    __syncthreads();
    for (int kk = 0; kk < 16; kk++) {
      cx<T> av[4], bv[4];
      for (int a = 0; a < 4; a++) av[a] = As[kk][tx + 16 * a];
      for (int b = 0; b < 4; b++) bv[b] = Bs[kk][ty + 16 * b];
      for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) acc[a][b] = acc[a][b] + av[a] * bv[b];
    }
    __syncthreads();
  }
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      int gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      if (gi < m && gj < n) {
        cx<T>* p = C + gi + (long long)gj * ldc;
        *p = *p - acc[a][b];
      }
    }
}

// ---- recursive panel (complex FP32) with cluster leaves ----
// Cluster size for the leaves of an N-row panel: 16 CTAs (non-portable) when
// the device schedules them, else 8; 0 if the rows do not fit.
static int leaf_cluster_size(int N, int smem_optin) {
  static int disabled = -1;
  if (disabled < 0) {
    const char* e = getenv("GBEM_LU_LEAF");
    disabled = (e && e[0] == '0') ? 1 : 0;
  }
  if (disabled) return 0;
  for (int CL : {16, 8}) {
    const size_t smem = (size_t)((N + CL - 1) / CL) * LEAF_STRIDE * sizeof(cx<float>);
    if (smem + 2048 > (size_t)smem_optin) continue;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, leaf_kernel) != cudaSuccess || smem + fa.sharedSizeBytes > (size_t)smem_optin ||
        allow_max_smem(leaf_kernel) != cudaSuccess)
      continue;
    if (CL > 8 && (cudaFuncSetAttribute(leaf_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
                   cudaFuncSetAttribute(leaf_kernel_reg<1, 1024>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                       cudaSuccess ||
                   cudaFuncSetAttribute(leaf_kernel_reg<1, 512>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                       cudaSuccess ||
                   cudaFuncSetAttribute(leaf_kernel_reg<2, 512>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                       cudaSuccess))
      continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, leaf_kernel, &cfg) == cudaSuccess && ncl >= 1) return CL;
    cudaGetLastError();
  }
  return 0;
}

// The lowest recursion level's U12 solve and update inside the right leaf
// (LeafArgs::fuse); GBEM_LU_FUSE=0 launches them as separate kernels.
static bool leaf_fusion() {
  static int f = -1;
  if (f < 0) {
    const char* e = getenv("GBEM_LU_FUSE");
    f = (e && e[0] == '0') ? 0 : 1;
  }
  return f == 1;
}

static cudaError_t leaf_launch_shape(const LeafArgs& la, int CL, int shape, cudaStream_t s) {
  if (la.fuse && la.Rr > 1024) return cudaErrorInvalidValue;  // register leaves only
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(shape == 1024 ? 1024 : 512);
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  if (la.Rr <= 1024 && shape == 1024) return cudaLaunchKernelEx(&cfg, leaf_kernel_reg<1, 1024>, la);
  if (la.Rr <= 512) return cudaLaunchKernelEx(&cfg, leaf_kernel_reg<1, 512>, la);
  if (la.Rr <= 1024) return cudaLaunchKernelEx(&cfg, leaf_kernel_reg<2, 512>, la);
  // rows in shared memory beyond two per thread
  cfg.dynamicSmemBytes = (size_t)la.Rr * LEAF_STRIDE * sizeof(cx<float>);
  return cudaLaunchKernelEx(&cfg, leaf_kernel, la);
}

// Tuning tables, per device: the register leaf's shape per 64-row bucket of
// rows per CTA, and the complex-FP32 panel width per 1024-row bucket of N.
static std::mutex g_tune_mu;
static std::vector<std::pair<long long, int>> g_leaf_tuned;   // (device * 1024 + bucket, threads)
static std::vector<std::pair<long long, int>> g_panel_tuned;  // (device * 1024 + bucket, width)

// Leaf shape autotuner.  For 512 < rows per CTA <= 1024 the leaf exists in
// two register shapes, 1024 threads x 1 row and 512 threads x 2 rows, whose
// order depends on the row count (45.7 vs 49.8 us for the latter at 960
// rows).  The first leaf of each 64-row bucket (per device) times both on a
// scratch copy of its panel columns -- the same data, the real launch
// geometry -- and the faster shape serves every later leaf of that bucket.
// GBEM_LU_LEAF_THREADS=512 or 1024 fixes the shape instead.
static int leaf_shape(const LeafArgs& la, int CL, cudaStream_t s) {
  if (la.Rr <= 512 || la.Rr > 1024) return 512;
  static int forced = -1;
  if (forced < 0) {
    const char* e = getenv("GBEM_LU_LEAF_THREADS");
    forced = e ? (atoi(e) == 1024 ? 1024 : 512) : 0;
  }
  if (forced) return forced;
  std::mutex& mu = g_tune_mu;
  std::vector<std::pair<long long, int>>& tuned = g_leaf_tuned;
  int dev = 0;
  cudaGetDevice(&dev);
  const long long key = (long long)dev * 1024 + (la.Rr - 1) / 64;
  {
    std::lock_guard<std::mutex> l(mu);
    for (auto& t : tuned)
      if (t.first == key) return t.second;
  }
  // scratch: the leaf's rows [c0, N) of the panel columns [pc0, pc1), with
  // its own pivots and info, indexed like the real matrix
  const long long rows = la.N - la.c0, cols = la.pc1 - la.pc0;
  cx<float>* scr = nullptr;
  int* sp = nullptr;
  int best = 512;
  float tbest = 1e30f;
  if (cudaMallocAsync((void**)&scr, sizeof(cx<float>) * (size_t)(rows * cols), s) == cudaSuccess &&
      cudaMallocAsync((void**)&sp, sizeof(int) * (size_t)(la.N + 1), s) == cudaSuccess) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    LeafArgs t = la;
    t.fuse = 0;  // the scratch holds rows c0.. only
    t.ld = rows;
    t.A = scr - la.c0 - (long long)la.pc0 * rows;  // element (r, c) of the panel at scr[(r - c0) + (c - pc0) rows]
    t.ipiv = sp;
    t.info = sp + la.N;
    for (int shape : {512, 1024}) {
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {
        cudaMemcpy2DAsync(scr, rows * sizeof(cx<float>), la.A + la.c0 + (long long)la.pc0 * la.ld,
                          la.ld * sizeof(cx<float>), rows * sizeof(cx<float>), cols, cudaMemcpyDeviceToDevice, s);
        cudaMemsetAsync(t.info, 0, sizeof(int), s);
        cudaEventRecord(e0, s);
        cudaError_t e = leaf_launch_shape(t, CL, shape, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        if (e != cudaSuccess) { ms = 1e30f; break; }
        cudaEventElapsedTime(&ms, e0, e1);
      }
      if (ms < tbest) { tbest = ms; best = shape; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  cudaGetLastError();
  if (scr) cudaFreeAsync(scr, s);
  if (sp) cudaFreeAsync(sp, s);
  std::lock_guard<std::mutex> l(mu);
  tuned.emplace_back(key, best);
  return best;
}

static cudaError_t leaf_launch(cx<float>* A, long long ld, int N, int c0, int w, int pc0, int pc1, int* ipiv, int* info,
                               int CL, cudaStream_t s, int fuse = 0) {
  const int m = N - c0;
  LeafArgs la;
  la.A = A; la.ld = ld; la.N = N; la.c0 = c0; la.w = w; la.Rr = (m + CL - 1) / CL; la.ipiv = ipiv; la.info = info;
  la.pc0 = pc0; la.pc1 = pc1; la.fuse = fuse;
  return leaf_launch_shape(la, CL, leaf_shape(la, CL, s), s);
}

// factor columns [c, c+w) of rows [c, N) inside the panel [pc0, pc1): left
// half, U12 = L11^{-1} A12, A22 -= L21 U12, right half.  The leaves apply
// their row interchanges to every column of the panel themselves.
// The U12 solves use the inverted 32 x 32 diagonal blocks of L (dinv, see
// trsm_kernel) wherever L11 is made of whole 32-blocks: the first solve that
// needs a block inverts it (made[] marks the blocks already in dinv).
struct DinvState {
  cx<float>* dinv = nullptr;
  std::vector<char> made;
};

static unsigned dinv_make_mask(DinvState* ds, int c, int h) {
  unsigned make = 0u;
  for (int b = 0; b < h / 32; b++) {
    char& m = ds->made[(c + 32 * b) / 32];
    if (!m) { make |= 1u << b; m = 1; }
  }
  return make;
}

static cudaError_t rec_panel(cx<float>* A, long long ld, int N, int c, int w, int pc0, int pc1, int* ipiv, int* info,
                             int CL, void* tcws, size_t tcb, DinvState* ds, cudaStream_t s, int* launches) {
  if (w <= LEAF_W) {
    ++*launches;
    return leaf_launch(A, ld, N, c, w, pc0, pc1, ipiv, info, CL, s);
  }
  const int h = ((w / 2 + LEAF_W - 1) / LEAF_W) * LEAF_W;
  cudaError_t e = rec_panel(A, ld, N, c, h, pc0, pc1, ipiv, info, CL, tcws, tcb, ds, s, launches);
  if (e != cudaSuccess) return e;
  const int wr = w - h, m2 = N - c - h;
  if (h == LEAF_W && wr <= LEAF_W && leaf_fusion() && (m2 + CL - 1) / CL <= 1024) {
    // lowest level: the right leaf applies the left one's U12 and update itself
    ++*launches;
    return leaf_launch(A, ld, N, c + h, wr, pc0, pc1, ipiv, info, CL, s, 1);
  }
  const bool dm = ds && h % 32 == 0 && c % 32 == 0;
  const unsigned make = dm ? dinv_make_mask(ds, c, h) : 0u;
  if (dm)
    launch_pdl(trsm_blocked<float>, dim3((wr + 31) / 32), dim3(256), (size_t)(2 * h + 32) * 33 * sizeof(cx<float>), s, 
        A, ld, c, h, c + h, c + w, ds->dinv, make);
  else
    launch_pdl(trsm_kernel<float>, dim3((wr + 31) / 32), dim3(256), (size_t)h * 33 * sizeof(cx<float>), s, A, ld, c, h, c + h, c + w);
  ++*launches;
  if (m2 > 0) {
    cx<float>* C = A + (c + h) + (long long)(c + h) * ld;
    const cx<float>* L21 = A + (c + h) + (long long)c * ld;
    const cx<float>* U12 = A + c + (long long)(c + h) * ld;
    // the wide updates of the upper levels on the tensor cores (split BF16)
    bool done = false;
    if (h >= 64 && m2 >= 128) {
      done = tc_gemm_update(C, ld, L21, ld, U12, ld, m2, wr, h, tcws, tcb, s, &e);
      if (e != cudaSuccess) return e;
      if (done) *launches += 3;
    }
    if (!done) {
      launch_pdl(gemm_simt<float>, dim3(dim3((m2 + 63) / 64, (wr + 63) / 64)), dim3(256), 0, s, C, ld, L21, ld, U12, ld, m2, wr, h);
      ++*launches;
    }
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return rec_panel(A, ld, N, c + h, wr, pc0, pc1, ipiv, info, CL, tcws, tcb, ds, s, launches);
}

template <typename T>
static gbem_status factor_impl(cx<T>* A, int N, int ld, int* d_ipiv, int* h_info, cudaStream_t s, void** ws,
                               size_t* ws_bytes, int force_w = 0);

// Panel width of the complex-FP32 LU with cluster leaves, per device and
// 1024-row bucket of N: 256 or 128, whichever factors a scratch copy of the
// bucket's first matrix faster (2 runs each; 1024 <= N <= 8192 -- at N = 15360
// 256 was measured best, and a scratch copy there would take 1.9 GB).
// GBEM_LU_PANEL=128 or 256 fixes it.
static int panel_width_c64(cx<float>* A, int N, int ld, cudaStream_t s, void** ws, size_t* ws_bytes) {
  static int forced = -1;
  if (forced < 0) {
    const char* e = getenv("GBEM_LU_PANEL");
    forced = e ? (atoi(e) == 128 ? 128 : 256) : 0;
  }
  if (forced) return forced;
  if (N < 1024 || N > 8192) return 256;
  int dev = 0;
  cudaGetDevice(&dev);
  const long long key = (long long)dev * 1024 + N / 1024;
  {
    std::lock_guard<std::mutex> l(g_tune_mu);
    for (auto& t : g_panel_tuned)
      if (t.first == key) return t.second;
  }
  int best = 256;
  cx<float>* scr = nullptr;
  int* sp = nullptr;
  if (cudaMallocAsync((void**)&scr, sizeof(cx<float>) * (size_t)N * N, s) == cudaSuccess &&
      cudaMallocAsync((void**)&sp, sizeof(int) * (size_t)N, s) == cudaSuccess) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float tbest = 1e30f;
    for (int w : {256, 128}) {
      float tw = 1e30f;
      for (int rep = 0; rep < 2; rep++) {
        int info = 0;
        cudaMemcpy2DAsync(scr, (size_t)N * sizeof(cx<float>), A, (size_t)ld * sizeof(cx<float>),
                          (size_t)N * sizeof(cx<float>), N, cudaMemcpyDeviceToDevice, s);
        cudaEventRecord(e0, s);
        const gbem_status st = factor_impl<float>(scr, N, N, sp, &info, s, ws, ws_bytes, w);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 1e30f;
        if (st == GBEM_OK) cudaEventElapsedTime(&ms, e0, e1);
        tw = std::min(tw, ms);
      }
      if (tw < tbest) { tbest = tw; best = w; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  cudaGetLastError();
  if (scr) cudaFreeAsync(scr, s);
  if (sp) cudaFreeAsync(sp, s);
  std::lock_guard<std::mutex> l(g_tune_mu);
  g_panel_tuned.emplace_back(key, best);
  return best;
}

template <typename T>
static gbem_status factor_impl(cx<T>* A, int N, int ld, int* d_ipiv, int* h_info, cudaStream_t s, void** ws,
                               size_t* ws_bytes, int force_w) {
  int dev = 0, nsm = 0, smem_optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t esz = sizeof(cx<T>);
  const size_t smem_cap = (size_t)smem_optin - 2048;
  // panel width: largest w whose panel rows fit the CTAs' shared memory
  int w = 256;
  int R = 0;
  for (;; w /= 2) {
    R = (N + nsm - 1) / nsm;
    if ((size_t)(R * panel_stride(w) + w) * esz <= smem_cap || w <= 8) break;
  }
  // complex FP32: recursive panels with cluster leaves where the leaf rows fit
  const int leaf_cl = sizeof(T) == 4 ? leaf_cluster_size(N, smem_optin) : 0;
  if (leaf_cl)
    w = force_w ? force_w
                : (sizeof(T) == 4 ? panel_width_c64((cx<float>*)A, N, ld, s, ws, ws_bytes) : 256);
  // programmatic dependent launch for the recursive-panel path only
  pdl_thread_on(leaf_cl != 0);
  struct PdlOff {
    ~PdlOff() { pdl_thread_on(false); }
  } pdl_off;
  if (w > N) w = std::max(1, N);
  R = std::max(R, 1);
  size_t smem = std::min((size_t)(R * panel_stride(w) + w) * esz, smem_cap);
  cudaError_t e = allow_max_smem(panel_kernel<T>);
  if (e != cudaSuccess) return cuda_status(e, "panel smem");
  int maxb = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, panel_kernel<T>, 512, smem);
  if (e != cudaSuccess || maxb < 1) return cuda_status(e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "panel occupancy");
  // workspace: stash + info + tensor-core scratch
  const int Gmax = nsm * maxb;
  size_t need = (size_t)2 * Gmax * w * esz + 2 * (size_t)w * esz + 2 * Gmax * sizeof(Cand) + 256;
  size_t tcb = 0;
  if (sizeof(T) == 4) tcb = tc_gemm_ws_bytes(N, N, w);
  const size_t dinv_bytes = (size_t)((N + 31) / 32) * 1024 * esz;
  const size_t swap_bytes = sizeof(int) * (4 * 256 + 16);
  size_t total = need + tcb + 1024 + dinv_bytes + 256 + swap_bytes + 256;
  if (*ws_bytes < total) {
    if (*ws) cudaFree(*ws);
    *ws = nullptr;
    *ws_bytes = 0;
    e = cudaMalloc(ws, total);
    if (e != cudaSuccess) return cuda_status(e, "LU workspace");
    *ws_bytes = total;
  }
  unsigned char* wp = (unsigned char*)*ws;
  Stash<T> st;
  st.cand_rows = (cx<T>*)wp; wp += (size_t)2 * Gmax * w * esz;
  st.diag_row = (cx<T>*)wp; wp += (size_t)2 * w * esz;
  st.cand = (Cand*)(((uintptr_t)wp + 15) & ~(uintptr_t)15); wp = (unsigned char*)(st.cand + 2 * Gmax);
  int* d_info = (int*)(((uintptr_t)wp + 15) & ~(uintptr_t)15); wp = (unsigned char*)(d_info + 4);
  void* tcws = (void*)(((uintptr_t)wp + 1023) & ~(uintptr_t)1023);
  cx<T>* dinv = (cx<T>*)(((uintptr_t)tcws + tcb + 255) & ~(uintptr_t)255);
  int* swap_mv = (int*)(((uintptr_t)((unsigned char*)dinv + dinv_bytes) + 255) & ~(uintptr_t)255);
  int* swap_n = swap_mv + 4 * 256;
  DinvState ds;
  ds.dinv = (cx<float>*)dinv;
  ds.made.assign((N + 31) / 32, 0);
  e = cudaMemsetAsync(d_info, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e, "info");
  // the U12 solves (outer and inside recursive panels) stage at most w rows
  // plus one inverted diagonal tile
  e = allow_max_smem(trsm_kernel<T>);
  if (e == cudaSuccess) e = allow_max_smem(trsm_blocked<T>);
  if (e != cudaSuccess) return cuda_status(e, "trsm smem");
  for (int c0 = 0; c0 < N; c0 += w) {
    const int wc = std::min(w, N - c0);
    const int m = N - c0;
    int G = std::min(Gmax, (m + R - 1) / R);
    if (!leaf_cl && G > 256) { set_error("LU panel: %d CTAs exceed the 256 candidate slots", G); return GBEM_ENOTSUP; }
    PanelArgs<T> pa;
    pa.A = A; pa.ld = ld; pa.N = N; pa.c0 = c0; pa.w = wc; pa.R = (m + G - 1) / G;
    pa.ipiv = d_ipiv; pa.info = d_info; pa.st = st;
    size_t sm = (size_t)(pa.R * panel_stride(wc) + wc) * esz;
    void* args[] = {&pa};
    {
      StatTimer tp(ST_PANEL, s);
      if (leaf_cl) {
        int nl = 0;
        e = rec_panel((cx<float>*)A, ld, N, c0, wc, c0, c0 + wc, d_ipiv, d_info, leaf_cl, tcws, tcb, &ds, s, &nl);
        stats_launch(ST_PANEL, nl);
        if (e != cudaSuccess) return cuda_status(e, "recursive panel");
      } else {
        stats_launch(ST_PANEL, 1);
        e = cudaLaunchCooperativeKernel((void*)panel_kernel<T>, dim3(G), dim3(512), args, sm, s);
        if (e != cudaSuccess) return cuda_status(e, "panel_kernel");
      }
      // interchanges to the left and right of the panel
      launch_pdl(swap_compose, dim3(1), dim3(256), 0, s, d_ipiv, c0, c0 + wc, swap_mv, swap_n);
      launch_pdl(swap_apply<T>, dim3((unsigned)((32LL * N + 255) / 256)), dim3(256), 0, s, A, ld, swap_mv, swap_n, 0, N, c0, c0 + wc);
      stats_launch(ST_PANEL, 2);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "row interchanges");
    }
    const int cb = c0 + wc;
    if (cb >= N) break;
    const int nrest = N - cb;
    const bool dm = wc % 32 == 0 && c0 % 32 == 0 && (size_t)(2 * wc + 32) * 33 * esz <= smem_cap;
    size_t tsm = (size_t)(dm ? 2 * wc + 32 : wc) * 33 * esz;
    // complex FP32 with a whole 256-row panel: U12 = L11^-1 A12 in two halves,
    // X1 = L11a^-1 B1, B2 -= L21 X1 on the tensor cores, X2 = L22^-1 B2 -- the
    // off-diagonal half of the solve's products leaves the FP32 pipes
    bool split = false;
    if (sizeof(T) == 4 && dm && leaf_cl && wc == 256) {
      StatTimer tt(ST_PANEL, s);
      const int h = wc / 2;
      const size_t hsm = (size_t)(2 * h + 32) * 33 * esz;
      // blocks the recursion left uninverted (the last one): inverted once
      // here rather than by every CTA of the wide solves below
      if (dinv_make_mask(&ds, c0, wc)) {
        launch_pdl(tri_inv_blocks<T>, dim3(wc / 32), dim3(256), 0, s, A, ld, c0, dinv);
        stats_launch(ST_PANEL);
      }
      launch_pdl(trsm_blocked<T>, dim3((nrest + 31) / 32), dim3(256), hsm, s, A, ld, c0, h, cb, N, dinv, 0u);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "trsm");
      stats_launch(ST_PANEL);
      cx<float>* B2 = (cx<float>*)(A + (c0 + h) + (long long)cb * ld);
      const cx<float>* L21h = (const cx<float>*)(A + (c0 + h) + (long long)c0 * ld);
      const cx<float>* X1 = (const cx<float>*)(A + c0 + (long long)cb * ld);
      if (tc_gemm_update(B2, ld, L21h, ld, X1, ld, h, nrest, h, tcws, tcb, s, &e)) {
        stats_launch(ST_PANEL, 3);
      } else {
        if (e != cudaSuccess) return cuda_status(e, "tensor-core update");
        launch_pdl(gemm_simt<float>, dim3(dim3((h + 63) / 64, (nrest + 63) / 64)), dim3(256), 0, s, B2, ld, L21h, ld, X1, ld, h, nrest, h);
        stats_launch(ST_PANEL);
      }
      launch_pdl(trsm_blocked<T>, dim3((nrest + 31) / 32), dim3(256), hsm, s, A, ld, c0 + h, h, cb, N, dinv, 0u);
      stats_launch(ST_PANEL);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "trsm");
      split = true;
    }
    if (!split) {
      StatTimer tt(ST_PANEL, s);
      unsigned make = 0u;
      if (dm && leaf_cl) {
        make = dinv_make_mask(&ds, c0, wc);  // blocks no recursive solve inverted yet
      } else if (dm) {
        // the grid panel has no recursive solves: invert the panel's blocks first
        launch_pdl(tri_inv_blocks<T>, dim3(wc / 32), dim3(256), 0, s, A, ld, c0, dinv);
        stats_launch(ST_PANEL);
      }
      stats_launch(ST_PANEL);
      if (dm)
        launch_pdl(trsm_blocked<T>, dim3((nrest + 31) / 32), dim3(256), tsm, s, A, ld, c0, wc, cb, N, dinv, make);
      else
        launch_pdl(trsm_kernel<T>, dim3((nrest + 31) / 32), dim3(256), tsm, s, A, ld, c0, wc, cb, N);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "trsm");
    }
    StatTimer tg(ST_GEMM, s);
    cx<T>* C = A + cb + (long long)cb * ld;
    const cx<T>* L21 = A + cb + (long long)c0 * ld;
    const cx<T>* U12 = A + c0 + (long long)cb * ld;
    bool done = false;
    if (sizeof(T) == 4) {
      done = tc_gemm_update((cx<float>*)C, ld, (const cx<float>*)L21, ld, (const cx<float>*)U12, ld, nrest, nrest, wc,
                            tcws, tcb, s, &e);
      if (e != cudaSuccess) return cuda_status(e, "tensor-core update");
      if (done) stats_launch(ST_GEMM, 3);
    }
    if (!done) {
      dim3 grid((nrest + 63) / 64, (nrest + 63) / 64);
      launch_pdl(gemm_simt<T>, dim3(grid), dim3(256), 0, s, C, ld, L21, ld, U12, ld, nrest, nrest, wc);
      stats_launch(ST_GEMM);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "gemm");
    }
  }
  e = cudaMemcpyAsync(h_info, d_info, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "LU");
  if (sizeof(T) == 4 && tc_gemm_error(true)) {
    set_error("LU: a bounded wait in the tensor-core update gave up");
    return GBEM_ETIMEOUT;
  }
  return GBEM_OK;
}

// The tuning tables as JSON (for the calling device), for reports.
std::string lu_tuning_json() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> l(g_tune_mu);
  std::string out = "{\"leaf_threads_by_rows_per_cta\": {";
  bool first = true;
  for (auto& t : g_leaf_tuned)
    if (t.first / 1024 == dev) {
      const long long b = t.first % 1024;
      out += (first ? "" : ", ") + std::string("\"") + std::to_string(64 * b + 1) + "-" + std::to_string(64 * b + 64) +
             "\": " + std::to_string(t.second);
      first = false;
    }
  out += "}, \"panel_width_by_N\": {";
  first = true;
  for (auto& t : g_panel_tuned)
    if (t.first / 1024 == dev) {
      const long long b = t.first % 1024;
      out += (first ? "" : ", ") + std::string("\"") + std::to_string(1024 * b) + "-" + std::to_string(1024 * b + 1023) +
             "\": " + std::to_string(t.second);
      first = false;
    }
  out += "}}";
  return out;
}

gbem_status lu_factor_device(void* dA, int N, int ld, int dtype, int* d_ipiv, int* h_info, cudaStream_t s, void** ws,
                             size_t* ws_bytes) {
  if (N <= 0 || ld < N) { set_error("lu_factor: bad size"); return GBEM_EINVAL; }
  if (dtype == GBEM_C128) return factor_impl<double>((cx<double>*)dA, N, ld, d_ipiv, h_info, s, ws, ws_bytes);
  if (dtype == GBEM_C64) return factor_impl<float>((cx<float>*)dA, N, ld, d_ipiv, h_info, s, ws, ws_bytes);
  set_error("lu_factor: dtype must be C128 or C64");
  return GBEM_EINVAL;
}

// ---------------------------------------------------------------------------
// triangular solves (forward with unit L, backward with U), blocked by 64
// ---------------------------------------------------------------------------
// B[perm[i]] -> Y[i]  (perm: final row order implied by ipiv)
template <typename T>
__global__ void gather_rows(const cx<T>* B, long long ldb, cx<T>* Y, long long ldy, const int* perm, int N, int nrhs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int r = 0; r < nrhs; r++) Y[i + r * ldy] = B[perm[i] + r * ldb];
}
template <typename T>
__global__ void scatter_rows(const cx<T>* Y, long long ldy, cx<T>* B, long long ldb, const int* perm, int N, int nrhs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int r = 0; r < nrhs; r++) B[perm[i] + r * ldb] = Y[i + r * ldy];
}

// solve the diagonal block [i0, i0+bs) in place; lower: unit L, forward;
// upper: U, backward; transposed variants use op(A) = A^T.
template <typename T, bool LOWER, bool TRANS>
__global__ void __launch_bounds__(256) diag_solve(const cx<T>* A, long long lda, cx<T>* X, long long ldx, int i0,
                                                   int bs, int nrhs) {
  constexpr int BSM = sizeof(T) == 4 ? 64 : 32;
  __shared__ cx<T> x[64][8];
  __shared__ cx<T> blk[BSM][BSM + 1];  // the diagonal block, staged once (coalesced)
  for (int q = threadIdx.x; q < bs * bs; q += blockDim.x) {
    int r = q % bs, c = q / bs;
    blk[r][c] = A[(i0 + r) + (long long)(i0 + c) * lda];
  }
  for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) x[q % bs][q / bs] = X[i0 + q % bs + (long long)(q / bs) * ldx];
  __syncthreads();
  for (int s = 0; s < bs; s++) {
    int k = (LOWER != TRANS) ? s : bs - 1 - s;  // forward for L or U^T, backward for U or L^T
    if (!LOWER) {
      if (threadIdx.x < nrhs) x[k][threadIdx.x] = cdiv(x[k][threadIdx.x], blk[k][k]);
      __syncthreads();
    }
    int rem = (LOWER != TRANS) ? bs - k - 1 : k;
    for (int q = threadIdx.x; q < rem * nrhs; q += blockDim.x) {
      int ii = (LOWER != TRANS) ? k + 1 + q % rem : q % rem;
      int rr = q / rem;
      cx<T> a = TRANS ? blk[k][ii] : blk[ii][k];
      x[ii][rr] = x[ii][rr] - a * x[k][rr];
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) X[i0 + q % bs + (long long)(q / bs) * ldx] = x[q % bs][q / bs];
}

// X[rows outside block] -= op(A)[rows, block] * X[block]
template <typename T, bool TRANS>
__global__ void __launch_bounds__(256) off_update(const cx<T>* A, long long lda, cx<T>* X, long long ldx, int i0, int bs,
                                                   int r0, int r1, int nrhs) {
  __shared__ cx<T> xb[64][8];
  for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) xb[q % bs][q / bs] = X[i0 + q % bs + (long long)(q / bs) * ldx];
  __syncthreads();
  int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  cx<T> acc[8];
  for (int r = 0; r < nrhs; r++) acc[r] = mk((T)0, (T)0);
  for (int k = 0; k < bs; k++) {
    cx<T> a = TRANS ? A[(i0 + k) + (long long)i * lda] : A[i + (long long)(i0 + k) * lda];
    for (int r = 0; r < nrhs; r++) acc[r] = acc[r] + a * xb[k][r];
  }
  for (int r = 0; r < nrhs; r++) X[i + (long long)r * ldx] = X[i + (long long)r * ldx] - acc[r];
}

// Inverses of the diagonal blocks of L (unit lower) or U (upper), one CTA
// per block: Dinv[k] = (A_kk)^{-1}, bs x bs column-major, block k at
// Dinv + k*bs*bs.  Solved as A_kk X = I column-parallel in shared memory.
template <typename T, bool LOWER>
__global__ void __launch_bounds__(256) diag_inverse(const cx<T>* A, long long lda, int N, int bs, cx<T>* Dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* blk = reinterpret_cast<cx<T>*>(smem_raw);  // [bs][bs+1] row-major
  cx<T>* X = blk + bs * (bs + 1);                     // [bs][bs+1]
  const int kb = blockIdx.x, i0 = kb * bs, n = min(bs, N - i0);
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
    int r = q % n, c = q / n;
    blk[r * (bs + 1) + c] = A[(i0 + r) + (long long)(i0 + c) * lda];
    X[r * (bs + 1) + c] = mk((T)(r == c ? 1 : 0), (T)0);
  }
  __syncthreads();
  for (int s = 0; s < n; s++) {
    int k = LOWER ? s : n - 1 - s;
    if (!LOWER) {
      for (int j = threadIdx.x; j < n; j += blockDim.x) X[k * (bs + 1) + j] = cdiv(X[k * (bs + 1) + j], blk[k * (bs + 1) + k]);
      __syncthreads();
    }
    int rem = LOWER ? n - k - 1 : k;
    for (int q = threadIdx.x; q < rem * n; q += blockDim.x) {
      int i = LOWER ? k + 1 + q % rem : q % rem, j = q / rem;
      X[i * (bs + 1) + j] = X[i * (bs + 1) + j] - blk[i * (bs + 1) + k] * X[k * (bs + 1) + j];
    }
    __syncthreads();
  }
  cx<T>* out = Dinv + (size_t)kb * bs * bs;
  for (int q = threadIdx.x; q < bs * bs; q += blockDim.x) {
    int r = q % bs, c = q / bs;
    out[r + (size_t)c * bs] = (r < n && c < n) ? X[r * (bs + 1) + c] : mk((T)0, (T)0);
  }
}

// Blocked triangular solve in one cooperative launch, one grid barrier per
// block.  Step s applies x_k (k = the s-th block in solve order) to the rows
// still unsolved: CTA 0 takes the rows of the next block k1 and at once solves
// that block from shared memory (x_k1 = Dinv_k1 (y_k1 - A(k1, k) x_k)), while
// the other CTAs update every row beyond k1.  CTA 0's operands for the next
// step (Dinv_k2 and A(k2 rows, k1 columns)) do not depend on x, so their
// cp.async copies into the second buffer are issued at the start of a step
// and land during its work and the grid barrier, off the critical path.
// Dynamic shared memory: 4 * bs * bs elements (bs <= 64, nrhs <= 8).
template <typename T, bool LOWER>
__global__ void __launch_bounds__(256) trsv_coop(const cx<T>* A, long long lda, int N, int bs, const cx<T>* Dinv,
                                                  cx<T>* Y, int nrhs) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* base = reinterpret_cast<cx<T>*>(smem_raw);
  // per buffer: Dinv of the block CTA 0 solves next (bs x bs, column-major)
  // and A(rows of that block, columns of the current one)
  cx<T>* const Dbuf[2] = {base, base + 2 * bs * bs};
  cx<T>* const Abuf[2] = {base + bs * bs, base + 3 * bs * bs};
  __shared__ cx<T> xs[64][8];                       // x of the block CTA 0 solved last
  __shared__ cx<T> rk[64][8];
  __shared__ cx<T> xk[64][8];                       // x_k for the general update
  const int nb = (N + bs - 1) / bs;
  const int tid = threadIdx.x, nt = blockDim.x, G = gridDim.x;
  const cx<T> zero = mk((T)0, (T)0);
  auto kb_of = [&](int s) { return LOWER ? s : nb - 1 - s; };
  auto n_of = [&](int k) { return min(bs, N - k * bs); };
  // CTA 0: Dbuf[b] <- Dinv[kd], Abuf[b] <- A(rows of block kr, columns of block kc), asynchronously
  auto stage = [&](int b, int kd, int kr, int kc) {
    const cx<T>* Dg = Dinv + (size_t)kd * bs * bs;
    const int nr_ = n_of(kr), nc_ = n_of(kc), r0_ = kr * bs, c0_ = kc * bs, bb = bs * bs;
    for (int q = tid; q < bb; q += nt) {
      const int r = q % bs, cc = q / bs;
      cp_async_cx(&Dbuf[b][q], Dg + q);
      if (r < nr_ && cc < nc_) cp_async_cx(&Abuf[b][q], &A[(r0_ + r) + (long long)(c0_ + cc) * lda]);
      else Abuf[b][q] = zero;
    }
    cp_async_commit();
  };
  if (blockIdx.x == 0) {
    // first block: x = Dinv y
    const int k = kb_of(0), i0 = k * bs, n = n_of(k);
    stage(0, k, k, k);
    for (int q = tid; q < n * nrhs; q += nt) rk[q % n][q / n] = ldcg_cx(Y + i0 + q % n + (long long)(q / n) * N);
    cp_async_wait_all();
    __syncthreads();
    for (int q = tid; q < n * nrhs; q += nt) {
      const int r = q % n, c = q / n;
      cx<T> acc = zero;
      for (int kk = 0; kk < n; kk++) acc = acc + Dbuf[0][r + kk * bs] * rk[kk][c];
      Y[i0 + r + (long long)c * N] = acc;
      xs[r][c] = acc;
    }
    __syncthreads();
    if (nb > 1) stage(1, kb_of(1), kb_of(1), k);
    __threadfence();
  }
  grid.sync();
  for (int s = 0; s + 1 < nb; s++) {
    const int k = kb_of(s), k1 = kb_of(s + 1);
    const int i0 = k * bs, n = n_of(k), i1 = k1 * bs, n1 = n_of(k1);
    if (blockIdx.x == 0) {
      const int cur = (s + 1) & 1;
      cp_async_wait_all();  // this step's operands
      __syncthreads();
      if (s + 2 < nb) stage(cur ^ 1, kb_of(s + 2), kb_of(s + 2), k1);  // the next step's, in flight meanwhile
      const cx<T>* D = Dbuf[cur];
      const cx<T>* Ab = Abuf[cur];
      // rows of k1: r = y - A(k1, k) x_k, then x_k1 = Dinv_k1 r
      for (int q = tid; q < n1 * nrhs; q += nt) {
        const int r = q % n1, c = q / n1;
        cx<T> acc = ldcg_cx(Y + i1 + r + (long long)c * N);
        for (int kk = 0; kk < n; kk++) acc = acc - Ab[r + kk * bs] * xs[kk][c];
        rk[r][c] = acc;
      }
      __syncthreads();
      for (int q = tid; q < n1 * nrhs; q += nt) {
        const int r = q % n1, c = q / n1;
        cx<T> acc = zero;
        for (int kk = 0; kk < n1; kk++) acc = acc + D[r + kk * bs] * rk[kk][c];
        Y[i1 + r + (long long)c * N] = acc;
        xs[r][c] = acc;
      }
      __syncthreads();
      __threadfence();
    }
    // rows beyond k1 (below it for L, above it for U), 4 threads per row
    const int r0 = LOWER ? i1 + n1 : 0, r1 = LOWER ? N : i1;
    if ((blockIdx.x != 0 || G == 1) && r1 > r0) {
      const int cb = G == 1 ? 0 : blockIdx.x - 1, GC = G == 1 ? 1 : G - 1;
      for (int q = tid; q < n * nrhs; q += nt) xk[q % n][q / n] = ldcg_cx(Y + i0 + q % n + (long long)(q / n) * N);
      __syncthreads();
      const int sub = tid & 3;
      const int nrows = r1 - r0;
      // the loop trip count is uniform over the CTA, so every lane reaches the shuffles
      for (int base0 = (cb * nt) >> 2; base0 < nrows; base0 += (GC * nt) >> 2) {
        const int base = base0 + (tid >> 2);
        const bool valid = base < nrows;
        const int i = r0 + (valid ? base : 0);
        cx<T> acc[8];
#pragma unroll
        for (int c = 0; c < 8; c++) acc[c] = zero;
        cx<T> a[16];
#pragma unroll
        for (int t = 0; t < 16; t++) {
          const int kk = sub + 4 * t;
          a[t] = (valid && kk < n) ? A[i + (long long)(i0 + kk) * lda] : zero;
        }
#pragma unroll
        for (int t = 0; t < 16; t++) {
          const int kk = sub + 4 * t;
          if (kk < n) {
#pragma unroll
            for (int c = 0; c < 8; c++)
              if (c < nrhs) acc[c] = acc[c] + a[t] * xk[kk][c];
          }
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
          if (c < nrhs) {  // nrhs is uniform: every lane takes the shuffles
            cx<T> v = acc[c];
            v.re += __shfl_xor_sync(0xffffffff, v.re, 1); v.im += __shfl_xor_sync(0xffffffff, v.im, 1);
            v.re += __shfl_xor_sync(0xffffffff, v.re, 2); v.im += __shfl_xor_sync(0xffffffff, v.im, 2);
            if (valid && sub == 0) Y[i + (long long)c * N] = ldcg_cx(Y + i + (long long)c * N) - v;
          }
        }
      }
      __threadfence();
    }
    grid.sync();
  }
}

// CTAs of the triangular solves: GBEM_TRSV_CTAS caps the grid (default: one
// per SM, fewer when N is small)
static int trsv_ctas() {
  static int c = -1;
  if (c < 0) {
    const char* e = getenv("GBEM_TRSV_CTAS");
    c = e ? std::max(0, atoi(e)) : 0;
  }
  return c;
}

template <typename T>
static gbem_status solve_impl(const cx<T>* A, int N, int ld, const int* d_perm, char trans, int nrhs, cx<T>* B, int ldb,
                              cx<T>* Y, cudaStream_t s) {
  const int bs = sizeof(T) == 4 ? 64 : 32;  // diagonal block staged in shared memory
  cudaError_t e;
  for (int r0 = 0; r0 < nrhs; r0 += 8) {
    int nr = std::min(8, nrhs - r0);
    cx<T>* Bc = B + (long long)r0 * ldb;
    if (trans == 'N') {
      gather_rows<T><<<(N + 255) / 256, 256, 0, s>>>(Bc, ldb, Y, N, d_perm, N, nr);
      const int nb = (N + bs - 1) / bs;
      cx<T>* Dinv = nullptr;
      e = cudaMallocAsync((void**)&Dinv, sizeof(cx<T>) * (size_t)nb * bs * bs * 2, s);
      if (e != cudaSuccess) return cuda_status(e, "solve workspace");
      cx<T>* DinvU = Dinv + (size_t)nb * bs * bs;
      size_t ism = sizeof(cx<T>) * 2 * bs * (bs + 1);
      allow_max_smem(diag_inverse<T, true>);
      allow_max_smem(diag_inverse<T, false>);
      diag_inverse<T, true><<<nb, 256, ism, s>>>(A, ld, N, bs, Dinv);
      diag_inverse<T, false><<<nb, 256, ism, s>>>(A, ld, N, bs, DinvU);
      int dev = 0, nsm = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      size_t dsm = sizeof(cx<T>) * 4 * bs * bs;
      allow_max_smem(trsv_coop<T, true>);
      allow_max_smem(trsv_coop<T, false>);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, trsv_coop<T, true>, 256, dsm);
      // 4 threads per row; one CTA per SM is enough to keep the reads in flight
      int G = std::max(1, std::min(nsm * std::max(per, 1), std::min(nsm, (4 * N + 255) / 256)));
      if (trsv_ctas() > 0) G = std::max(1, std::min(G, trsv_ctas()));
      int Nn = N, bsn = bs, nrn = nr;
      const cx<T>* Ac = A;
      long long ldl = ld;
      void* argsL[] = {(void*)&Ac, (void*)&ldl, (void*)&Nn, (void*)&bsn, (void*)&Dinv, (void*)&Y, (void*)&nrn};
      e = cudaLaunchCooperativeKernel((void*)trsv_coop<T, true>, dim3(G), dim3(256), argsL, dsm, s);
      if (e != cudaSuccess) return cuda_status(e, "trsv lower");
      void* argsU[] = {(void*)&Ac, (void*)&ldl, (void*)&Nn, (void*)&bsn, (void*)&DinvU, (void*)&Y, (void*)&nrn};
      e = cudaLaunchCooperativeKernel((void*)trsv_coop<T, false>, dim3(G), dim3(256), argsU, dsm, s);
      if (e != cudaSuccess) return cuda_status(e, "trsv upper");
      cudaFreeAsync(Dinv, s);
      stats_launch(ST_SOLVE, 5);
      e = cudaMemcpy2DAsync(Bc, (size_t)ldb * sizeof(cx<T>), Y, (size_t)N * sizeof(cx<T>), (size_t)N * sizeof(cx<T>), nr,
                            cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(e, "solve copy");
    } else {
      // A^T x = b with A = P^T L U: U^T z = b, L^T y = z, x = P^T y
      e = cudaMemcpy2DAsync(Y, (size_t)N * sizeof(cx<T>), Bc, (size_t)ldb * sizeof(cx<T>), (size_t)N * sizeof(cx<T>), nr,
                            cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(e, "solve copy");
      for (int i0 = 0; i0 < N; i0 += bs) {
        int b = std::min(bs, N - i0);
        diag_solve<T, false, true><<<1, 256, 0, s>>>(A, ld, Y, N, i0, b, nr);
        if (i0 + b < N) off_update<T, true><<<(N - i0 - b + 255) / 256, 256, 0, s>>>(A, ld, Y, N, i0, b, i0 + b, N, nr);
      }
      for (int i0 = ((N - 1) / bs) * bs; i0 >= 0; i0 -= bs) {
        int b = std::min(bs, N - i0);
        diag_solve<T, true, true><<<1, 256, 0, s>>>(A, ld, Y, N, i0, b, nr);
        if (i0 > 0) off_update<T, true><<<(i0 + 255) / 256, 256, 0, s>>>(A, ld, Y, N, i0, b, 0, i0, nr);
      }
      scatter_rows<T><<<(N + 255) / 256, 256, 0, s>>>(Y, N, Bc, ldb, d_perm, N, nr);
      stats_launch(ST_SOLVE, 2 + 4 * ((N + bs - 1) / bs));
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "solve");
  }
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// Solve with many right-hand sides (X = A^-1 B, trans 'N', nrhs ~ N): the
// permutation, then per diagonal block the block inverse applied from
// shared memory and a GEMM update of the rows still to be solved.  Used for
// Tr[M^-1 dM] (the force and torque integrand of scuff-cas3D), where the
// right-hand side is a whole block column of dM.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) block_apply(const cx<T>* Dinv, int bs, int n, cx<T>* Y, long long ldy, int i0,
                                                   int nrhs) {
  __shared__ cx<T> y[64][17];
  const int c0 = blockIdx.x * 16;
  for (int q = threadIdx.x; q < n * 16; q += blockDim.x) {
    const int r = q % n, c = q / n;
    y[r][c] = c0 + c < nrhs ? Y[i0 + r + (long long)(c0 + c) * ldy] : mk((T)0, (T)0);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < n * 16; q += blockDim.x) {
    const int r = q % n, c = q / n;
    if (c0 + c >= nrhs) continue;
    cx<T> acc = mk((T)0, (T)0);
    for (int kk = 0; kk < n; kk++) acc = acc + Dinv[r + (size_t)kk * bs] * y[kk][c];
    Y[i0 + r + (long long)(c0 + c) * ldy] = acc;
  }
}

template <typename T>
static gbem_status solve_many_impl(const cx<T>* A, int N, int ld, const int* d_perm, int nrhs, cx<T>* B, int ldb,
                                   cudaStream_t s) {
  const int bs = sizeof(T) == 4 ? 64 : 32;
  const int nb = (N + bs - 1) / bs;
  cx<T>* Y = nullptr;
  cx<T>* Dinv = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&Y, sizeof(cx<T>) * (size_t)N * nrhs, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&Dinv, sizeof(cx<T>) * (size_t)nb * bs * bs * 2, s);
  if (e != cudaSuccess) return cuda_status(e, "solve workspace");
  cx<T>* DinvU = Dinv + (size_t)nb * bs * bs;
  gather_rows<T><<<(N + 255) / 256, 256, 0, s>>>(B, ldb, Y, N, d_perm, N, nrhs);
  const size_t ism = sizeof(cx<T>) * 2 * bs * (bs + 1);
  allow_max_smem(diag_inverse<T, true>);
  allow_max_smem(diag_inverse<T, false>);
  diag_inverse<T, true><<<nb, 256, ism, s>>>(A, ld, N, bs, Dinv);
  diag_inverse<T, false><<<nb, 256, ism, s>>>(A, ld, N, bs, DinvU);
  const dim3 ga((nrhs + 15) / 16);
  for (int b = 0; b < nb; b++) {  // forward: unit L
    const int i0 = b * bs, n = std::min(bs, N - i0), m = N - i0 - n;
    block_apply<T><<<ga, 256, 0, s>>>(Dinv + (size_t)b * bs * bs, bs, n, Y, N, i0, nrhs);
    if (m > 0)
      gemm_simt<T><<<dim3((m + 63) / 64, (nrhs + 63) / 64), 256, 0, s>>>(Y + i0 + n, N, A + (i0 + n) + (long long)i0 * ld,
                                                                        ld, Y + i0, N, m, nrhs, n);
  }
  for (int b = nb - 1; b >= 0; b--) {  // backward: U
    const int i0 = b * bs, n = std::min(bs, N - i0);
    block_apply<T><<<ga, 256, 0, s>>>(DinvU + (size_t)b * bs * bs, bs, n, Y, N, i0, nrhs);
    if (i0 > 0)
      gemm_simt<T><<<dim3((i0 + 63) / 64, (nrhs + 63) / 64), 256, 0, s>>>(Y, N, A + (long long)i0 * ld, ld, Y + i0, N,
                                                                         i0, nrhs, n);
  }
  stats_launch(ST_SOLVE, 3 + 4 * nb);
  e = cudaMemcpy2DAsync(B, (size_t)ldb * sizeof(cx<T>), Y, (size_t)N * sizeof(cx<T>), (size_t)N * sizeof(cx<T>), nrhs,
                        cudaMemcpyDeviceToDevice, s);
  cudaFreeAsync(Dinv, s);
  cudaFreeAsync(Y, s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? GBEM_OK : cuda_status(e, "solve (many right-hand sides)");
}

gbem_status lu_solve_many_device(const void* dA, int N, int ld, int dtype, const int* d_perm, int nrhs, void* dB, int ldb,
                                 cudaStream_t s) {
  if (dtype == GBEM_C128)
    return solve_many_impl<double>((const cx<double>*)dA, N, ld, d_perm, nrhs, (cx<double>*)dB, ldb, s);
  if (dtype == GBEM_C64)
    return solve_many_impl<float>((const cx<float>*)dA, N, ld, d_perm, nrhs, (cx<float>*)dB, ldb, s);
  set_error("lu_solve: dtype must be C128 or C64");
  return GBEM_EINVAL;
}

// B <- conj(B): A^H x = b is A^T conj(x) = conj(b) (zgetrs with Trans = 'C')
template <typename T>
__global__ void conj_cols(cx<T>* B, long long ldb, int N, int nrhs) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)N * nrhs) return;
  cx<T>* b = B + (q % N) + (q / N) * ldb;
  b->im = -b->im;
}

template <typename T>
static gbem_status solve_any(const cx<T>* A, int N, int ld, const int* d_perm, char trans, int nrhs, cx<T>* B, int ldb,
                             cx<T>* Y, cudaStream_t s) {
  if (trans != 'C') return solve_impl<T>(A, N, ld, d_perm, trans, nrhs, B, ldb, Y, s);
  const unsigned nb = (unsigned)(((long long)N * nrhs + 255) / 256);
  conj_cols<T><<<nb, 256, 0, s>>>(B, ldb, N, nrhs);
  gbem_status st = solve_impl<T>(A, N, ld, d_perm, 'T', nrhs, B, ldb, Y, s);
  if (st != GBEM_OK) return st;
  conj_cols<T><<<nb, 256, 0, s>>>(B, ldb, N, nrhs);
  stats_launch(ST_SOLVE, 2);
  return cuda_status(cudaGetLastError(), "solve conj");
}

gbem_status lu_solve_device(const void* dA, int N, int ld, int dtype, const int* d_perm, char trans, int nrhs, void* dB,
                            int ldb, void* dY, cudaStream_t s) {
  if (trans != 'N' && trans != 'T' && trans != 'C') {
    set_error("lu_solve: trans must be 'N', 'T' or 'C'");
    return GBEM_EINVAL;
  }
  if (dtype == GBEM_C128)
    return solve_any<double>((const cx<double>*)dA, N, ld, d_perm, trans, nrhs, (cx<double>*)dB, ldb, (cx<double>*)dY, s);
  if (dtype == GBEM_C64)
    return solve_any<float>((const cx<float>*)dA, N, ld, d_perm, trans, nrhs, (cx<float>*)dB, ldb, (cx<float>*)dY, s);
  set_error("lu_solve: dtype must be C128 or C64");
  return GBEM_EINVAL;
}

// ---------------------------------------------------------------------------
// FP64 residual R = B - A X for a C64 or C128 matrix A and C128 X, B
// ---------------------------------------------------------------------------
template <typename TA>
__global__ void __launch_bounds__(128) residual_partial(const cx<TA>* A, long long lda, const cx<double>* X, long long ldx,
                                                        int N, int nrhs, int cchunk, cx<double>* part) {
  __shared__ cx<double> xs[128][8];
  const int i = blockIdx.x * 128 + threadIdx.x;
  const int c0 = blockIdx.y * cchunk, c1 = min(N, c0 + cchunk);
  cx<double> acc[8];
  for (int r = 0; r < 8; r++) acc[r] = mk(0.0, 0.0);
  for (int j0 = c0; j0 < c1; j0 += 128) {
    int nj = min(128, c1 - j0);
    __syncthreads();
    for (int q = threadIdx.x; q < nj * nrhs; q += 128) xs[q % nj][q / nj] = X[(j0 + q % nj) + (long long)(q / nj) * ldx];
    __syncthreads();
    if (i < N)
      for (int j = 0; j < nj; j++) {
        cx<TA> a = A[i + (long long)(j0 + j) * lda];
        cx<double> ad = mk((double)a.re, (double)a.im);
        for (int r = 0; r < nrhs; r++) acc[r] = acc[r] + ad * xs[j][r];
      }
  }
  if (i < N)
    for (int r = 0; r < nrhs; r++) part[((size_t)blockIdx.y * nrhs + r) * N + i] = acc[r];
}

// Double-float residual for a complex-FP32 matrix: every product A_ij * x_j
// with x_j = xh + xl (two FP32 pieces of the FP64 value) is formed as an
// exact FP32 pair (p, fma(a, xh, -p)) plus the small term a * xl, and summed
// with Knuth's two-sum into a (hi, lo) FP32 accumulator; every 64 columns the
// pair is folded into an FP64 partial sum.  The rounding left is ~64 * 2^-48
// of the partial sums, far below the refinement tolerance, at FP32 rates.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
  float s = __fadd_rn(hi, p);
  float bb = __fadd_rn(s, -hi);
  float err = __fadd_rn(__fadd_rn(hi, -__fadd_rn(s, -bb)), __fadd_rn(p, -bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

template <int NR>
__global__ void __launch_bounds__(128) residual_partial_df(const cx<float>* A, long long lda, const cx<double>* X,
                                                           long long ldx, int N, int cchunk, cx<double>* part) {
  __shared__ float4 xs[64][NR];  // (re_hi, re_lo, im_hi, im_lo)
  const int i = blockIdx.x * 128 + threadIdx.x;
  const int c0 = blockIdx.y * cchunk, c1 = min(N, c0 + cchunk);
  double accr[NR], acci[NR];
  for (int r = 0; r < NR; r++) accr[r] = acci[r] = 0.0;
  const cx<float>* Ai = A + (i < N ? i : 0);
  for (int j0 = c0; j0 < c1; j0 += 64) {
    const int nj = min(64, c1 - j0);
    __syncthreads();
    for (int q = threadIdx.x; q < nj * NR; q += 128) {
      int j = q % nj, r = q / nj;
      cx<double> x = X[(j0 + j) + (long long)r * ldx];
      float rh = (float)x.re, ih = (float)x.im;
      xs[j][r] = make_float4(rh, (float)(x.re - (double)rh), ih, (float)(x.im - (double)ih));
    }
    __syncthreads();
    float hr[NR], lr[NR], hi_[NR], li[NR];
    for (int r = 0; r < NR; r++) hr[r] = lr[r] = hi_[r] = li[r] = 0.f;
    if (i < N) {
#pragma unroll 4
      for (int j = 0; j < nj; j++) {
        const cx<float> a = Ai[(long long)(j0 + j) * lda];
#pragma unroll
        for (int r = 0; r < NR; r++) {
          const float4 x = xs[j][r];
          // real part: a.re*xr - a.im*xi
          float p1 = __fmul_rn(a.re, x.x), e1 = __fmaf_rn(a.re, x.x, -p1);
          float p2 = __fmul_rn(-a.im, x.z), e2 = __fmaf_rn(-a.im, x.z, -p2);
          two_sum_acc(hr[r], lr[r], p1);
          two_sum_acc(hr[r], lr[r], p2);
          lr[r] = __fadd_rn(lr[r], __fadd_rn(e1, e2));
          lr[r] = __fmaf_rn(a.re, x.y, lr[r]);
          lr[r] = __fmaf_rn(-a.im, x.w, lr[r]);
          // imaginary part: a.re*xi + a.im*xr
          float p3 = __fmul_rn(a.re, x.z), e3 = __fmaf_rn(a.re, x.z, -p3);
          float p4 = __fmul_rn(a.im, x.x), e4 = __fmaf_rn(a.im, x.x, -p4);
          two_sum_acc(hi_[r], li[r], p3);
          two_sum_acc(hi_[r], li[r], p4);
          li[r] = __fadd_rn(li[r], __fadd_rn(e3, e4));
          li[r] = __fmaf_rn(a.re, x.w, li[r]);
          li[r] = __fmaf_rn(a.im, x.y, li[r]);
        }
      }
    }
    for (int r = 0; r < NR; r++) {
      accr[r] += (double)hr[r] + (double)lr[r];
      acci[r] += (double)hi_[r] + (double)li[r];
    }
  }
  if (i < N)
    for (int r = 0; r < NR; r++) part[((size_t)blockIdx.y * NR + r) * N + i] = mk(accr[r], acci[r]);
}

__global__ void residual_finish(const cx<double>* B, long long ldb, const cx<double>* part, int nsplit, int N, int nrhs,
                                cx<double>* R, long long ldr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int r = 0; r < nrhs; r++) {
    cx<double> s = B[i + (long long)r * ldb];
    for (int p = 0; p < nsplit; p++) s = s - part[((size_t)p * nrhs + r) * N + i];
    R[i + (long long)r * ldr] = s;
  }
}

gbem_status residual_device(const void* dA, int lda, int dtype, int N, const double* dX, int ldx, const double* dB,
                            int ldb, int nrhs, double* dR, int ldr, void* part, cudaStream_t s) {
  // column splits: more partial sums put more rows x chunks in flight
  // (GBEM_RESID_SPLIT, at most RESID_MAX_SPLIT)
  static int nsplit = -1;
  if (nsplit < 0) {
    const char* ev = getenv("GBEM_RESID_SPLIT");
    nsplit = ev ? std::max(1, std::min(RESID_MAX_SPLIT, atoi(ev))) : 24;
  }
  int cchunk = (N + nsplit - 1) / nsplit;
  cudaError_t e;
  for (int r0 = 0; r0 < nrhs; r0 += 8) {
    int nr = std::min(8, nrhs - r0);
    dim3 grid((N + 127) / 128, nsplit);
    const cx<double>* X = (const cx<double>*)dX + (long long)r0 * ldx;
    if (dtype == GBEM_C64) {
      const cx<float>* Af = (const cx<float>*)dA;
      cx<double>* P = (cx<double>*)part;
      switch (nr) {
        case 1: residual_partial_df<1><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 2: residual_partial_df<2><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 3: residual_partial_df<3><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 4: residual_partial_df<4><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 5: residual_partial_df<5><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 6: residual_partial_df<6><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        case 7: residual_partial_df<7><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
        default: residual_partial_df<8><<<grid, 128, 0, s>>>(Af, lda, X, ldx, N, cchunk, P); break;
      }
    } else
      residual_partial<double><<<grid, 128, 0, s>>>((const cx<double>*)dA, lda, X, ldx, N, nr, cchunk, (cx<double>*)part);
    stats_launch(ST_RESID, 2);
    residual_finish<<<(N + 255) / 256, 256, 0, s>>>((const cx<double>*)dB + (long long)r0 * ldb, ldb, (cx<double>*)part,
                                                   nsplit, N, nr, (cx<double>*)dR + (long long)r0 * ldr, ldr);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "residual");
  }
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// LU solve that allocates no device memory: its workspace is a file-scope
// device array reserved when this module loads on a device.  Every call on a
// device shares that device's array and leaves its last contents there;
// nothing in it has to start at zero, because each call writes every scratch
// byte before reading it.  Calls that overlap in time on one device race on
// the array; the call synchronises the matrix's stream before it returns.
// ---------------------------------------------------------------------------
static constexpr size_t kSolveScratchBytes = (size_t)16 << 20;
static __device__ __align__(256) unsigned char g_solve_scratch[kSolveScratchBytes];
static constexpr int kMaxDevices = 64;
static void* g_solve_scratch_ptr[kMaxDevices];  // device address per ordinal, set on first use
static std::mutex g_solve_scratch_mu;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// bytes of scratch one chunk of <= 8 right-hand sides needs: the chunk's
// columns, the permuted copy Y, and the inverses of the diagonal blocks
static size_t solve_scratch_need(int N, int dtype) {
  const size_t es = dtype == GBEM_C64 ? 8 : 16;
  const size_t bs = dtype == GBEM_C64 ? 64 : 32;
  const size_t nb = ((size_t)N + bs - 1) / bs;
  return 2 * align256((size_t)N * 8 * es) + align256(2 * nb * bs * bs * es);
}

// one chunk (nr <= 8 columns) of A X = B, 'N' form, with caller-provided Y and
// Dinv; the same kernels and launch shapes as solve_impl
template <typename T>
static gbem_status solve_chunk_n(const cx<T>* A, int N, int ld, const int* d_perm, int nr, cx<T>* Bc, int ldb, cx<T>* Y,
                                 cx<T>* Dinv, cudaStream_t s) {
  const int bs = sizeof(T) == 4 ? 64 : 32;
  const int nb = (N + bs - 1) / bs;
  cudaError_t e;
  gather_rows<T><<<(N + 255) / 256, 256, 0, s>>>(Bc, ldb, Y, N, d_perm, N, nr);
  cx<T>* DinvU = Dinv + (size_t)nb * bs * bs;
  size_t ism = sizeof(cx<T>) * 2 * bs * (bs + 1);
  allow_max_smem(diag_inverse<T, true>);
  allow_max_smem(diag_inverse<T, false>);
  diag_inverse<T, true><<<nb, 256, ism, s>>>(A, ld, N, bs, Dinv);
  diag_inverse<T, false><<<nb, 256, ism, s>>>(A, ld, N, bs, DinvU);
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  size_t dsm = sizeof(cx<T>) * 4 * bs * bs;
  allow_max_smem(trsv_coop<T, true>);
  allow_max_smem(trsv_coop<T, false>);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, trsv_coop<T, true>, 256, dsm);
  int G = std::max(1, std::min(nsm * std::max(per, 1), std::min(nsm, (4 * N + 255) / 256)));
  int Nn = N, bsn = bs, nrn = nr;
  const cx<T>* Ac = A;
  long long ldl = ld;
  void* argsL[] = {(void*)&Ac, (void*)&ldl, (void*)&Nn, (void*)&bsn, (void*)&Dinv, (void*)&Y, (void*)&nrn};
  e = cudaLaunchCooperativeKernel((void*)trsv_coop<T, true>, dim3(G), dim3(256), argsL, dsm, s);
  if (e != cudaSuccess) return cuda_status(e, "trsv lower");
  void* argsU[] = {(void*)&Ac, (void*)&ldl, (void*)&Nn, (void*)&bsn, (void*)&DinvU, (void*)&Y, (void*)&nrn};
  e = cudaLaunchCooperativeKernel((void*)trsv_coop<T, false>, dim3(G), dim3(256), argsU, dsm, s);
  if (e != cudaSuccess) return cuda_status(e, "trsv upper");
  stats_launch(ST_SOLVE, 5);
  e = cudaMemcpy2DAsync(Bc, (size_t)ldb * sizeof(cx<T>), Y, (size_t)N * sizeof(cx<T>), (size_t)N * sizeof(cx<T>), nr,
                        cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "solve copy");
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "solve");
  return GBEM_OK;
}

template <typename T>
static gbem_status solve_static_impl(const cx<T>* A, int N, int ld, const int* d_perm, char trans, int nrhs, cx<T>* hB,
                                     int ldb, unsigned char* scratch, cudaStream_t s) {
  const size_t es = sizeof(cx<T>);
  cx<T>* Bd = (cx<T>*)scratch;
  cx<T>* Y = (cx<T>*)(scratch + align256((size_t)N * 8 * es));
  cx<T>* Dinv = (cx<T>*)(scratch + 2 * align256((size_t)N * 8 * es));
  gbem_status st = GBEM_OK;
  for (int r0 = 0; r0 < nrhs && st == GBEM_OK; r0 += 8) {
    const int nr = std::min(8, nrhs - r0);
    cx<T>* hc = hB + (long long)r0 * ldb;
    cudaError_t e = cudaMemcpy2DAsync(Bd, (size_t)N * es, hc, (size_t)ldb * es, (size_t)N * es, nr,
                                      cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { st = cuda_status(e, "solve upload"); break; }
    st = trans == 'N' ? solve_chunk_n<T>(A, N, ld, d_perm, nr, Bd, N, Y, Dinv, s)
                      : solve_any<T>(A, N, ld, d_perm, trans, nr, Bd, N, Y, s);  // 'T'/'C' allocate nothing
    if (st != GBEM_OK) break;
    e = cudaMemcpy2DAsync(hc, (size_t)ldb * es, Bd, (size_t)N * es, (size_t)N * es, nr, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "solve download");
  }
  // whatever happened, nothing of this call may still be queued on the shared
  // scratch array when it returns: the first error is kept
  cudaError_t es2 = cudaStreamSynchronize(s);
  if (st == GBEM_OK && es2 != cudaSuccess) st = cuda_status(es2, "solve");
  return st;
}

gbem_status lu_solve_static_scratch(const void* dA, int N, int ld, int dtype, const int* d_perm, char trans, int nrhs,
                                    void* hB, int ldb, cudaStream_t s) {
  if (trans != 'N' && trans != 'T' && trans != 'C') {
    set_error("gbem_lu_solve_noalloc: trans must be 'N', 'T' or 'C'");
    return GBEM_EINVAL;
  }
  if (dtype != GBEM_C128 && dtype != GBEM_C64) {
    set_error("gbem_lu_solve_noalloc: only complex128 and complex64 matrices are supported (a real F64 factor is "
              "solved through a complex128 copy of the whole matrix, which the static scratch cannot hold); use "
              "gbem_lu_solve for F64 matrices");
    return GBEM_EINVAL;
  }
  const size_t need = solve_scratch_need(N, dtype);
  if (need > kSolveScratchBytes) {
    set_error("gbem_lu_solve_noalloc: N = %d needs %zu bytes of scratch; the static scratch holds %zu bytes "
              "(N <= %d for complex128, N <= %d for complex64)",
              N, need, kSolveScratchBytes, lu_solve_noalloc_max_n(GBEM_C128), lu_solve_noalloc_max_n(GBEM_C64));
    return GBEM_EINVAL;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) { set_error("gbem_lu_solve_noalloc: device ordinal %d out of range", dev); return GBEM_EINVAL; }
  void* scratch = nullptr;
  {
    // first call on this device (with it current): look up the array's address
    std::lock_guard<std::mutex> l(g_solve_scratch_mu);
    if (!g_solve_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress((void**)&p, g_solve_scratch);
      if (e != cudaSuccess) return cuda_status(e, "gbem_lu_solve_noalloc: cudaGetSymbolAddress of the scratch array");
      g_solve_scratch_ptr[dev] = p;
    }
    scratch = g_solve_scratch_ptr[dev];
  }
  if (dtype == GBEM_C128)
    return solve_static_impl<double>((const cx<double>*)dA, N, ld, d_perm, trans, nrhs, (cx<double>*)hB, ldb,
                                     (unsigned char*)scratch, s);
  return solve_static_impl<float>((const cx<float>*)dA, N, ld, d_perm, trans, nrhs, (cx<float>*)hB, ldb,
                                  (unsigned char*)scratch, s);
}

// largest N whose solve fits the static scratch
int lu_solve_noalloc_max_n(int dtype) {
  int lo = 0, hi = 1 << 24;
  while (lo < hi) {
    int mid = lo + (hi - lo + 1) / 2;
    if (solve_scratch_need(mid, dtype) <= kSolveScratchBytes) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace gbem
