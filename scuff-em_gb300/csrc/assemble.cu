// assemble.cu -- BEM matrix assembly on the GPU (replaces
// RWGGeometry::AssembleBEMMatrix, AssembleBEMMatrix.cc:684-765, and the
// GetSurfaceSurfaceInteractions / GetEdgeEdgeInteractions /
// GetPanelPanelInteractions stack below it for compact geometries).
//
// Kernels
//  fippi_kernel   once per geometry: the frequency-independent static
//                 integrals of every near panel pair (FP64).
//  self_kernel    per frequency: common-triangle pairs (FP64, Taylor-Duffy
//                 reduction to 1-D).
//  near_kernel    per frequency: every other pair with rRel <= 4 (FP64,
//                 desingularised 6x6 rule + static table, or high-order rule
//                 in the short-wavelength regime).
//  tile_kernel<T> per frequency: one CTA per tile of TE x TE edge pairs.
//                 Computes the 6x6-rule bilinear moments of every panel pair
//                 the tile touches once (T = float for the mixed form,
//                 double for the plain form), forms the up-to-9 (Qa,Qb)
//                 combinations, and writes the tile's matrix entries (and
//                 the mirrored tile) with coalesced stores.  Each edge-pair
//                 entry gathers its four panel-pair contributions from
//                 per-(edge pair, P/M side) slots in shared memory, so the
//                 sum is deterministic and needs no atomics.
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {

// ---------------------------------------------------------------------------
// quadrature rules in constant memory
// ---------------------------------------------------------------------------
// LO rule: the 13-digit values of libs/libTriInt/TCR.cc:83-91 (order 4).
__constant__ double c_lo64[18];
__constant__ float c_lo32[18];
static const double h_lo[18] = {
    0.0915762135098, 0.0915762135098, 0.0549758718276, 0.8168475729805, 0.0915762135098, 0.0549758718276,
    0.0915762135098, 0.8168475729805, 0.0549758718276, 0.1081030181681, 0.4459484909160, 0.1116907948390,
    0.4459484909160, 0.1081030181681, 0.1116907948390, 0.4459484909160, 0.4459484909160, 0.1116907948390};
constexpr int HO_N = 11;                 // collapsed Gauss rule, degree 20
__constant__ double c_ho[3 * HO_N * HO_N];
constexpr int NT_SELF = 16;              // 1-D rule of the common-triangle reduction
constexpr int N_FIP = 12;                // rules of the static near-pair integrals
__constant__ double c_gx16[NT_SELF], c_gw16[NT_SELF], c_gx12[N_FIP], c_gw12[N_FIP];

static void gauss01(int n, double* x, double* w) {
  for (int i = 0; i < n; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[i] = 0.5 * (1 - z);
    w[i] = 1.0 / ((1 - z * z) * pp * pp);
  }
}

static gbem_status init_rules() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && done[dev]) return GBEM_OK;
  float lo32[18];
  for (int i = 0; i < 18; i++) lo32[i] = (float)h_lo[i];
  double x[HO_N], w[HO_N], ho[3 * HO_N * HO_N];
  gauss01(HO_N, x, w);
  int k = 0;
  for (int i = 0; i < HO_N; i++)
    for (int j = 0; j < HO_N; j++) {
      ho[k++] = x[i] * (1.0 - x[j]);
      ho[k++] = x[i] * x[j];
      ho[k++] = w[i] * w[j] * x[i];
    }
  double gx16[NT_SELF], gw16[NT_SELF], gx12[N_FIP], gw12[N_FIP];
  gauss01(NT_SELF, gx16, gw16);
  gauss01(N_FIP, gx12, gw12);
  cudaError_t e = cudaMemcpyToSymbol(c_lo64, h_lo, sizeof h_lo);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_lo32, lo32, sizeof lo32);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ho, ho, sizeof ho);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gx16, gx16, sizeof gx16);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gw16, gw16, sizeof gw16);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gx12, gx12, sizeof gx12);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gw12, gw12, sizeof gw12);
  if (e != cudaSuccess) return cuda_status(e, "copy quadrature rules");
  if (dev < 64) done[dev] = true;
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// device-side geometry
// ---------------------------------------------------------------------------
struct DevEdgeBlock {
  int e0, ne, np, pad;
  int panels[PMAX];
  int8_t hl[3 * PMAX];
  int8_t hs[3 * PMAX];
};

struct DevNear {
  int pa, pb;
  int ncv;
  int perm_a[3], perm_b[3];  // common-vertices-first order -> mesh order
  double rmax;
};

struct DevBlock {
  int nrows = 0, ncols = 0, ntiles = 0, nnear = 0, nself = 0, nother = 0;
  DevEdgeBlock* rows = nullptr;
  DevEdgeBlock* cols = nullptr;
  int2* tiles = nullptr;
  double* elen_a = nullptr;
  double* elen_b = nullptr;
  int* nptr = nullptr;
  int* ncol = nullptr;
  int* nidx = nullptr;
  DevNear* near = nullptr;
  int* self_list = nullptr;
  int* other_list = nullptr;
  Fippi* fippi = nullptr;     // per near pair (unused slots for self pairs)
  double* nearval = nullptr;  // 27 complex per near pair
};

template <typename Tp>
static cudaError_t dupload(Tp** d, const Tp* h, size_t n) {
  if (n == 0) { *d = nullptr; return cudaSuccess; }
  cudaError_t e = cudaMalloc((void**)d, n * sizeof(Tp));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h, n * sizeof(Tp), cudaMemcpyHostToDevice);
}

static DevEdgeBlock pack_block(const EdgeBlock& b) {
  DevEdgeBlock d;
  memset(&d, 0, sizeof d);
  d.e0 = b.e0; d.ne = b.ne; d.np = (int)b.panels.size();
  for (int i = 0; i < d.np; i++) d.panels[i] = b.panels[i];
  for (int i = 0; i < 3 * d.np; i++) { d.hl[i] = b.he_local[i]; d.hs[i] = b.he_side[i]; }
  return d;
}

gbem_status upload_geometry(Geometry* g) {
  if (g->d_pv) return GBEM_OK;
  cudaError_t e = cudaSetDevice(g->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  gbem_status st = init_rules();
  if (st != GBEM_OK) return st;
  std::vector<double> pv(9 * (size_t)g->np_total), pc(4 * (size_t)g->np_total);
  for (const Surface& s : g->S)
    for (int p = 0; p < s.np; p++) {
      size_t gp = s.panel_offset + p;
      for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) pv[9 * gp + 3 * i + c] = s.V[3 * s.PV[3 * p + i] + c];
      for (int c = 0; c < 3; c++) pc[4 * gp + c] = s.cen[3 * p + c];
      pc[4 * gp + 3] = s.rad[p];
    }
  e = dupload(&g->d_pv, pv.data(), pv.size());
  if (e == cudaSuccess) e = dupload(&g->d_pc, pc.data(), pc.size());
  if (e != cudaSuccess) return cuda_status(e, "upload panels");
  for (const Block& b : g->blocks) {
    DevBlock* db = new DevBlock();
    g->dblocks.push_back(db);
    std::vector<DevEdgeBlock> rows, cols;
    for (auto& eb : b.rows) rows.push_back(pack_block(eb));
    for (auto& eb : b.cols) cols.push_back(pack_block(eb));
    db->nrows = (int)rows.size(); db->ncols = (int)cols.size(); db->ntiles = (int)b.tiles.size();
    e = dupload(&db->rows, rows.data(), rows.size());
    if (e == cudaSuccess) e = dupload(&db->cols, cols.data(), cols.size());
    if (e == cudaSuccess) e = dupload(&db->tiles, b.tiles.data(), b.tiles.size());
    if (e == cudaSuccess) e = dupload(&db->elen_a, g->S[b.sa].elen.data(), g->S[b.sa].elen.size());
    if (e == cudaSuccess) e = dupload(&db->elen_b, g->S[b.sb].elen.data(), g->S[b.sb].elen.size());
    if (e == cudaSuccess) e = dupload(&db->nptr, b.near_ptr.data(), b.near_ptr.size());
    if (e == cudaSuccess) e = dupload(&db->ncol, b.near_col.data(), b.near_col.size());
    if (e == cudaSuccess) e = dupload(&db->nidx, b.near_idx.data(), b.near_idx.size());
    std::vector<DevNear> dn;
    std::vector<int> self_l, other_l[3];
    for (size_t i = 0; i < b.near.size(); i++) {
      const NearPair& n = b.near[i];
      DevNear d;
      d.pa = n.pa; d.pb = n.pb; d.ncv = n.ncv; d.rmax = n.rmax;
      for (int j = 0; j < 3; j++) { d.perm_a[j] = n.perm_a[j]; d.perm_b[j] = n.perm_b[j]; }
      dn.push_back(d);
      if (n.ncv == 3) self_l.push_back((int)i); else other_l[n.ncv].push_back((int)i);
    }
    std::vector<int> others;
    for (int c = 0; c < 3; c++) others.insert(others.end(), other_l[c].begin(), other_l[c].end());
    db->nnear = (int)dn.size(); db->nself = (int)self_l.size(); db->nother = (int)others.size();
    if (e == cudaSuccess) e = dupload(&db->near, dn.data(), dn.size());
    if (e == cudaSuccess) e = dupload(&db->self_list, self_l.data(), self_l.size());
    if (e == cudaSuccess) e = dupload(&db->other_list, others.data(), others.size());
    if (e == cudaSuccess && db->nnear) e = cudaMalloc((void**)&db->fippi, sizeof(Fippi) * db->nnear);
    if (e == cudaSuccess && db->nnear) e = cudaMalloc((void**)&db->nearval, sizeof(double) * 54 * db->nnear);
    if (e != cudaSuccess) return cuda_status(e, "upload blocks");
  }
  return GBEM_OK;
}

void free_geometry_device(Geometry* g) {
  cudaFree(g->d_pv); cudaFree(g->d_pc);
  g->d_pv = g->d_pc = nullptr;
  for (DevBlock* db : g->dblocks) {
    cudaFree(db->rows); cudaFree(db->cols); cudaFree(db->tiles); cudaFree(db->elen_a); cudaFree(db->elen_b);
    cudaFree(db->nptr); cudaFree(db->ncol); cudaFree(db->nidx); cudaFree(db->near); cudaFree(db->self_list);
    cudaFree(db->other_list); cudaFree(db->fippi); cudaFree(db->nearval);
    delete db;
  }
  g->dblocks.clear();
}

// ---------------------------------------------------------------------------
// per-frequency region data of a block
// ---------------------------------------------------------------------------
struct RegionArgs {
  int nreg;
  cx<double> k[2];     // wavenumber per common region
  cx<double> pf1[2];   // +-i mu omega   (SurfaceSurfaceInteractions.cc:165-176)
  cx<double> pfc[2];   // (-+i k) / (i k) : multiplies H1 (GC[1] carries 1/(ik))
  cx<double> pf3[2];   // -+i eps omega
};


// ---------------------------------------------------------------------------
// static near-pair table (once per geometry)
// ---------------------------------------------------------------------------
__global__ void fippi_kernel(const DevNear* near, const int* list, int n, const double* pv, Fippi* out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int i = list[t];
  DevNear d = near[i];
  double Va[9], Vb[9];
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  Fippi F;
  if (d.ncv == 0) {
    fippi_far(Va, Vb, c_gx12, c_gw12, N_FIP, &F);
  } else {
    fippi_touch(d.ncv, Va, Vb, d.perm_a, d.perm_b, c_gx12, c_gw12, N_FIP, &F);
  }
  out[i] = F;
}

// ---------------------------------------------------------------------------
// per-frequency near pairs
// ---------------------------------------------------------------------------
__device__ void store_near(double* dst, int ja, int jb, cx<double> kk, cx<double> kn, cx<double> nn) {
  double* o = dst + 6 * (3 * ja + jb);
  o[0] += kk.re; o[1] += kk.im; o[2] += kn.re; o[3] += kn.im; o[4] += nn.re; o[5] += nn.im;
}

// one warp per common-triangle pair: the 6*NT_SELF outer points are split
// over the lanes and the moments reduced with shuffles
__global__ void __launch_bounds__(128) self_kernel(const DevNear* near, const int* list, int n, const double* pv,
                                                   RegionArgs ra, double* nearval) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;  // whole warps exit together
  int i = list[warp];
  DevNear d = near[i];
  double V[9];
  for (int c = 0; c < 9; c++) V[c] = pv[9 * (size_t)d.pa + c];
  double* dst = nearval + 54 * (size_t)i;
  // lane q < 9 accumulates combination q = 3 ja + jb: KK (re, im), KN (zero), NN (re, im)
  double acc0 = 0.0, acc1 = 0.0, acc4 = 0.0, acc5 = 0.0;
  for (int r = 0; r < ra.nreg; r++) {
    cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    cx<double> MG[9], MP[9];
    self_moments(V, k, c_gx16, c_gw16, NT_SELF, MG, lane, 32);
    for (int m = 0; m < 9; m++) {
      for (int o = 16; o > 0; o >>= 1) {
        MG[m].re += __shfl_xor_sync(0xffffffff, MG[m].re, o);
        MG[m].im += __shfl_xor_sync(0xffffffff, MG[m].im, o);
      }
      MP[m] = mk(0.0, 0.0);
    }
    cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
    if (lane < 9) {
      int ja = lane / 3, jb = lane % 3;
      double c[9], dd[9];
      combo_coeffs(V, V, ja, jb, c, dd);
      cx<double> H0, H1;
      combine(MG, MP, c, dd, m4ok2, &H0, &H1);
      cx<double> v0 = ra.pf1[r] * H0, v2 = ra.pf3[r] * H0;
      acc0 += v0.re; acc1 += v0.im;
      acc4 += v2.re; acc5 += v2.im;
    }
  }
  if (lane < 9) {
    double* o = dst + 6 * lane;
    o[0] = acc0; o[1] = acc1; o[2] = 0.0; o[3] = 0.0; o[4] = acc4; o[5] = acc5;
  }
}

__global__ void near_kernel(const DevNear* near, const int* list, int n, const double* pv, const Fippi* fippi,
                            RegionArgs ra, double* nearval, int* status) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int i = list[t];
  DevNear d = near[i];
  double Va[9], Vb[9];
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  double* dst = nearval + 54 * (size_t)i;
  for (int c = 0; c < 54; c++) dst[c] = 0.0;
  const Fippi& F = fippi[i];  // read where used: keeps 33 doubles out of registers
  for (int r = 0; r < ra.nreg; r++) {
    cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    // short-wavelength test of PanelPanelInteractions.cc:416-418
    cx<double> kr = mk(k.re * d.rmax, k.im * d.rmax);
    bool sw = hypot(kr.re, kr.im) > M_PI;
    cx<double> MG[9], MP[9];
    bool desing = false;
    if (!sw) {
      pair_moments<double, 1>(g, k, c_lo64, 6, MG, MP);
      add_taylor_terms(F, k, MG, MP);
      desing = true;
    } else if (d.ncv == 0) {
      pair_moments<double, 0>(g, k, c_ho, HO_N * HO_N, MG, MP);
    } else {
      // touching pair in the short-wavelength regime: td_touch_kernel adds
      // this region's full-kernel Taylor-Duffy values after this kernel
      continue;
    }
    cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
    VecMoments<double> vm;
    vec_moments(g, MG, MP, &vm);
    for (int ja = 0; ja < 3; ja++)
      for (int jb = 0; jb < 3; jb++) {
        cx<double> H0, H1;
        vec_combine(g, vm, ja, jb, m4ok2, &H0, &H1);
        if (desing) H1 = H1 + mk(-0.079577471545947667884 * htimes_rm3(F, Va, Vb, ja, jb), 0.0);
        store_near(dst, ja, jb, ra.pf1[r] * H0, ra.pfc[r] * H1, ra.pf3[r] * H0);
      }
  }
}

// One warp per touching pair (ncv = 1, 2) in the short-wavelength regime
// (|k rmax| > pi, PanelPanelInteractions.cc:416-418): the Duffy points are
// split over the lanes, the 9 G moments and 10 H1 moments reduced with
// shuffles, and lanes 0..8 add the nine (Qa,Qb) combinations.
constexpr int N_TD = 12;  // Gauss points per Duffy dimension
__global__ void __launch_bounds__(128) td_touch_kernel(const DevNear* near, const int* list, int n, const double* pv,
                                                       RegionArgs ra, double* nearval) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;  // whole warps exit together
  const int i = list[warp];
  const DevNear d = near[i];
  if (d.ncv < 1 || d.ncv > 2) return;
  double Va[9], Vb[9];
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  double* dst = nearval + 54 * (size_t)i;
  for (int r = 0; r < ra.nreg; r++) {
    const cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    if (!(hypot(k.re * d.rmax, k.im * d.rmax) > M_PI)) continue;  // near_kernel's desingularised branch
    cx<double> MG[9], T[10];
    td_touch(d.ncv, Va, Vb, d.perm_a, d.perm_b, k, c_gx12, c_gw12, N_TD, lane, 32, MG, T);
    for (int m = 0; m < 9; m++)
      for (int o = 16; o > 0; o >>= 1) {
        MG[m].re += __shfl_xor_sync(0xffffffff, MG[m].re, o);
        MG[m].im += __shfl_xor_sync(0xffffffff, MG[m].im, o);
      }
    for (int m = 0; m < 10; m++)
      for (int o = 16; o > 0; o >>= 1) {
        T[m].re += __shfl_xor_sync(0xffffffff, T[m].re, o);
        T[m].im += __shfl_xor_sync(0xffffffff, T[m].im, o);
      }
    if (lane < 9) {
      const int ja = lane / 3, jb = lane % 3;
      cx<double> MP[9];
      for (int m = 0; m < 9; m++) MP[m] = mk(0.0, 0.0);
      VecMoments<double> vm;
      vec_moments(g, MG, MP, &vm);
      cx<double> H0, H1unused;
      vec_combine(g, vm, ja, jb, cdiv(mk(-4.0, 0.0), k * k), &H0, &H1unused);
      const cx<double> H1 = td_h1(Va, Vb, T, ja, jb);
      store_near(dst, ja, jb, ra.pf1[r] * H0, ra.pfc[r] * H1, ra.pf3[r] * H0);
    }
  }
}

// ---------------------------------------------------------------------------
// far-field tile kernel
// ---------------------------------------------------------------------------
struct TileArgs {
  const DevEdgeBlock* rows;
  const DevEdgeBlock* cols;
  const int2* tiles;
  const double* pv;
  const double* pc;
  const double* elen_a;
  const double* elen_b;
  const int* nptr;
  const int* ncol;
  const int* nidx;
  const double* nearval;
  int row_panel_offset;
  int bpe_a, bpe_b;
  int row_off, col_off;    // where entry (row edge, col edge) of the block goes
  int mrow_off, mcol_off;  // where its mirror (col edge, row edge) goes
  int passes;              // bit 0: write the block, bit 1: write the mirror
  int sym;
  void* out;
  long long ld;
};

template <typename T> __device__ __forceinline__ const T* lo_rule();
template <> __device__ __forceinline__ const float* lo_rule<float>() { return c_lo32; }
template <> __device__ __forceinline__ const double* lo_rule<double>() { return c_lo64; }

// relative distance with the reference's operation order and no FMA
// contraction (AssessPanelPair.cc:160-166)
__device__ __forceinline__ bool is_far(const double* ca, const double* cb, double ra, double rb) {
  double rmax = fmax(ra, rb);
  double dc = __dsub_rn(ca[0], cb[0]);
  double r2 = __dmul_rn(dc, dc);
  dc = __dsub_rn(ca[1], cb[1]);
  r2 = __dadd_rn(r2, __dmul_rn(dc, dc));
  dc = __dsub_rn(ca[2], cb[2]);
  r2 = __dadd_rn(r2, __dmul_rn(dc, dc));
  return __ddiv_rn(__dsqrt_rn(r2), rmax) > 4.0;
}

template <typename T, int NC>
__global__ void __launch_bounds__(256) tile_kernel(TileArgs a, RegionArgs ra) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* slots = reinterpret_cast<cx<T>*>(smem_raw);  // [TE][TE][4][NC]
  constexpr int PVN = sizeof(T) == 4 ? 1 : 9;  // the FP32 kernel keeps FP32 geometry only
  __shared__ double s_pv[2][PMAX][PVN];
  __shared__ double s_pc[2][PMAX][4];
  __shared__ int8_t s_hl[2][3 * PMAX], s_hs[2][3 * PMAX];
  __shared__ int s_gp[2][PMAX];
  __shared__ float s_ev[2][PMAX][6];  // FP32 edge vectors V1-V0, V2-V0
  __shared__ float s_cf[2][PMAX][4];  // FP32 centroid and radius (pre-check of rRel)
  __shared__ float s_v0[2][PMAX][6];  // V0 as FP32 (hi, lo) pairs: D0 to FP32 relative accuracy
  __shared__ cx<float> s_rk[2], s_rm4[2], s_rp1[2], s_rpc[2], s_rp3[2];  // per-region FP32 constants
  __shared__ int s_live[2];
  __shared__ T s_el[2][TE];  // edge lengths of the tile's rows and columns

  const int2 tile = a.tiles[blockIdx.x];
  const DevEdgeBlock* RB = a.rows + tile.x;
  const DevEdgeBlock* CB = a.cols + tile.y;
  const int PR = RB->np, PC = CB->np, NR = RB->ne, NCc = CB->ne;
  if constexpr (sizeof(T) == 8) {
    for (int q = threadIdx.x; q < PR * 9; q += blockDim.x) s_pv[0][q / 9][q % 9] = a.pv[9 * (size_t)RB->panels[q / 9] + q % 9];
    for (int q = threadIdx.x; q < PC * 9; q += blockDim.x) s_pv[1][q / 9][q % 9] = a.pv[9 * (size_t)CB->panels[q / 9] + q % 9];
  }
  for (int q = threadIdx.x; q < PR * 4; q += blockDim.x) s_pc[0][q / 4][q % 4] = a.pc[4 * (size_t)RB->panels[q / 4] + q % 4];
  for (int q = threadIdx.x; q < PC * 4; q += blockDim.x) s_pc[1][q / 4][q % 4] = a.pc[4 * (size_t)CB->panels[q / 4] + q % 4];
  for (int q = threadIdx.x; q < 3 * PR; q += blockDim.x) { s_hl[0][q] = RB->hl[q]; s_hs[0][q] = RB->hs[q]; }
  for (int q = threadIdx.x; q < 3 * PC; q += blockDim.x) { s_hl[1][q] = CB->hl[q]; s_hs[1][q] = CB->hs[q]; }
  for (int q = threadIdx.x; q < PR; q += blockDim.x) s_gp[0][q] = RB->panels[q];
  for (int q = threadIdx.x; q < PC; q += blockDim.x) s_gp[1][q] = CB->panels[q];
  __syncthreads();
  for (int q = threadIdx.x; q < 2 * PMAX; q += blockDim.x) {
    const int side = q / PMAX, p = q % PMAX;
    if (p >= (side ? PC : PR)) continue;
    const double* V = a.pv + 9 * (size_t)(side ? CB->panels[p] : RB->panels[p]);
    for (int c = 0; c < 3; c++) { s_ev[side][p][c] = (float)(V[3 + c] - V[c]); s_ev[side][p][3 + c] = (float)(V[6 + c] - V[c]); }
    for (int c = 0; c < 4; c++) s_cf[side][p][c] = (float)s_pc[side][p][c];
    for (int c = 0; c < 3; c++) {
      const float hi = (float)V[c];
      s_v0[side][p][c] = hi;
      s_v0[side][p][3 + c] = (float)(V[c] - (double)hi);
    }
  }
  for (int q = threadIdx.x; q < 2 * TE; q += blockDim.x) {
    const int side = q / TE, e = q % TE;
    if (e < (side ? NCc : NR)) s_el[side][e] = (T)(side ? a.elen_b[CB->e0 + e] : a.elen_a[RB->e0 + e]);
  }
  if (threadIdx.x < 2) {
    // region constants in FP32, formed once per CTA in FP64
    const int r = threadIdx.x;
    const cx<double> kd = r < ra.nreg ? ra.k[r] : mk(0.0, 0.0);
    const bool live = !(kd.re == 0.0 && kd.im == 0.0);
    s_live[r] = live;
    const cx<double> m4d = live ? cdiv(mk(-4.0, 0.0), kd * kd) : mk(0.0, 0.0);
    s_rk[r] = mk((float)kd.re, (float)kd.im);
    s_rm4[r] = mk((float)m4d.re, (float)m4d.im);
    s_rp1[r] = live ? mk((float)ra.pf1[r].re, (float)ra.pf1[r].im) : mk(0.0f, 0.0f);
    s_rpc[r] = live ? mk((float)ra.pfc[r].re, (float)ra.pfc[r].im) : mk(0.0f, 0.0f);
    s_rp3[r] = live ? mk((float)ra.pf3[r].re, (float)ra.pf3[r].im) : mk(0.0f, 0.0f);
  }
  __syncthreads();

  const T* rule = lo_rule<T>();
  for (int q = threadIdx.x; q < PR * PC; q += blockDim.x) {
    const int ia = q / PC, ib = q - ia * PC;
    const double* Va = s_pv[0][ia];
    const double* Vb = s_pv[1][ib];
    int la[3], lb[3], sa[3], sb[3];
    for (int j = 0; j < 3; j++) {
      la[j] = s_hl[0][3 * ia + j]; sa[j] = s_hs[0][3 * ia + j];
      lb[j] = s_hl[1][3 * ib + j]; sb[j] = s_hs[1][3 * ib + j];
    }
    // rRel > 4 decides the 6x6 rule; an FP32 estimate settles all but the
    // pairs within 1e-4 of the threshold, which take the exact FP64 test
    const float dx = s_cf[0][ia][0] - s_cf[1][ib][0], dy = s_cf[0][ia][1] - s_cf[1][ib][1],
                dz = s_cf[0][ia][2] - s_cf[1][ib][2];
    const float d2f = dx * dx + dy * dy + dz * dz, rmf = fmaxf(s_cf[0][ia][3], s_cf[1][ib][3]);
    bool far;
    if (d2f > 16.0008f * rmf * rmf) far = true;
    else if (d2f < 15.9992f * rmf * rmf) far = false;
    else far = is_far(s_pc[0][ia], s_pc[1][ib], s_pc[0][ia][3], s_pc[1][ib][3]);
    if (far) {
      PairGeom<T> g;
      for (int c = 0; c < 3; c++) {
        if constexpr (sizeof(T) == 4)
          g.D0[c] = (s_v0[0][ia][c] - s_v0[1][ib][c]) + (s_v0[0][ia][3 + c] - s_v0[1][ib][3 + c]);
        else
          g.D0[c] = (T)(Va[c] - Vb[c]);
        if constexpr (sizeof(T) == 4) {
          g.Aa[c] = s_ev[0][ia][c]; g.Ba[c] = s_ev[0][ia][3 + c];
          g.Ab[c] = s_ev[1][ib][c]; g.Bb[c] = s_ev[1][ib][3 + c];
        } else {
          g.Aa[c] = (T)(Va[3 + c] - Va[c]); g.Ba[c] = (T)(Va[6 + c] - Va[c]);
          g.Ab[c] = (T)(Vb[3 + c] - Vb[c]); g.Bb[c] = (T)(Vb[6 + c] - Vb[c]);
        }
      }
      if constexpr (sizeof(T) == 4) {
        // FP32: per region, the 9+9 moments in vector form, then every needed
        // (Qa,Qb) from them (vec_combine); the slot takes the first region's
        // value and adds the second's (one writer per slot: deterministic)
        constexpr int R2 = NC == 1 ? 1 : 2;
        for (int r = 0; r < R2; r++) {
          const bool live = s_live[r];
          VecMoments<T> vm;
          const cx<T> m4 = s_rm4[r], p1 = s_rp1[r], pc = s_rpc[r], p3 = s_rp3[r];
          if (live) {
            cx<T> MG[9], MP[9];
            pair_moments<T, 0>(g, s_rk[r], rule, 6, MG, MP);
            vec_moments(g, MG, MP, &vm);
          }
          for (int ja = 0; ja < 3; ja++) {
            if (la[ja] < 0) continue;
            for (int jb = 0; jb < 3; jb++) {
              if (lb[jb] < 0) continue;
              cx<T> v0 = mk((T)0, (T)0), v1 = v0, v2 = v0;
              if (live) {
                cx<T> H0, H1;
                vec_combine(g, vm, ja, jb, m4, &H0, &H1);
                v0 = p1 * H0;
                v1 = pc * H1;
                v2 = p3 * H0;
              }
              cx<T>* sl = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
              if (r == 0) {
                sl[0] = v0;
                if (NC > 1) sl[1] = v1;
                if (NC > 2) sl[2] = v2;
              } else {
                sl[0] = sl[0] + v0;
                if (NC > 1) sl[1] = sl[1] + v1;
                if (NC > 2) sl[2] = sl[2] + v2;
              }
            }
          }
        }
      } else {
      bool first = true;
      for (int r = 0; r < ra.nreg; r++) {
        cx<double> kd = ra.k[r];
        if (kd.re == 0.0 && kd.im == 0.0) continue;
        cx<T> k = mk((T)kd.re, (T)kd.im);
        cx<T> MG[9], MP[9];
        pair_moments<T, 0>(g, k, rule, 6, MG, MP);
        cx<double> m4ok2d = cdiv(mk(-4.0, 0.0), kd * kd);
        cx<T> m4ok2 = mk((T)m4ok2d.re, (T)m4ok2d.im);
        cx<T> p1 = mk((T)ra.pf1[r].re, (T)ra.pf1[r].im), pc = mk((T)ra.pfc[r].re, (T)ra.pfc[r].im),
              p3 = mk((T)ra.pf3[r].re, (T)ra.pf3[r].im);
        for (int ja = 0; ja < 3; ja++) {
          if (la[ja] < 0) continue;
          for (int jb = 0; jb < 3; jb++) {
            if (lb[jb] < 0) continue;
            double cd[9], dd[9];
            combo_coeffs(Va, Vb, ja, jb, cd, dd);
            T c[9], d[9];
            for (int m = 0; m < 9; m++) { c[m] = (T)cd[m]; d[m] = (T)dd[m]; }
            cx<T> H0, H1;
            combine(MG, MP, c, d, m4ok2, &H0, &H1);
            cx<T>* s = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
            cx<T> v0 = p1 * H0;
            if (first) s[0] = v0; else s[0] = s[0] + v0;
            if (NC > 1) { cx<T> v1 = pc * H1; if (first) s[1] = v1; else s[1] = s[1] + v1; }
            if (NC > 2) { cx<T> v2 = p3 * H0; if (first) s[2] = v2; else s[2] = s[2] + v2; }
          }
        }
        first = false;
      }
      if (first) {  // every common region has k = 0: zero contribution
        for (int ja = 0; ja < 3; ja++)
          for (int jb = 0; jb < 3; jb++)
            if (la[ja] >= 0 && lb[jb] >= 0) {
              cx<T>* s = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
              for (int c = 0; c < NC; c++) s[c] = mk((T)0, (T)0);
            }
      }
      }
    } else {
      // near pair: values precomputed in FP64 by self_kernel / near_kernel
      int gpa = s_gp[0][ia], gpb = s_gp[1][ib];
      int row = gpa - a.row_panel_offset, hit = -1;
      for (int e = a.nptr[row]; e < a.nptr[row + 1]; e++)
        if (a.ncol[e] == gpb) { hit = a.nidx[e]; break; }
      if (hit < 0) continue;  // cannot happen: every rRel<=4 pair is listed
      const double* nv = a.nearval + 54 * (size_t)(hit >> 1);
      const bool tr = hit & 1;
      for (int ja = 0; ja < 3; ja++) {
        if (la[ja] < 0) continue;
        for (int jb = 0; jb < 3; jb++) {
          if (lb[jb] < 0) continue;
          const double* v = nv + 6 * (tr ? (3 * jb + ja) : (3 * ja + jb));
          cx<T>* s = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
          s[0] = mk((T)v[0], (T)v[1]);
          if (NC > 1) s[1] = mk((T)v[2], (T)v[3]);
          if (NC > 2) s[2] = mk((T)v[4], (T)v[5]);
        }
      }
    }
  }
  __syncthreads();

  // entries: sum of the four P/M contributions times La Lb
  cx<T>* out = reinterpret_cast<cx<T>*>(a.out);
  const long long ld = a.ld;
  // A diagonal tile of a symmetric block writes its upper triangle and
  // mirrors it, so the matrix is exactly symmetric (AssembleBEMMatrix.cc:753-758).
  const bool diag = a.sym && tile.x == tile.y;
  for (int pass = 0; pass < 2; pass++) {
    if (!(a.passes & (1 << pass))) continue;
    for (int q = threadIdx.x; q < NR * NCc; q += blockDim.x) {
      int i, j;
      if (pass == 0) { i = q % NR; j = q / NR; } else { j = q % NCc; i = q / NCc; }
      if (diag && (pass == 0 ? i > j : i >= j)) continue;
      const cx<T>* s = slots + (size_t)(i * TE + j) * 4 * NC;
      cx<T> v[3];
      for (int c = 0; c < NC; c++) v[c] = (s[c] - s[NC + c]) - (s[2 * NC + c] - s[3 * NC + c]);
      T L;
      if constexpr (sizeof(T) == 4) L = s_el[0][i] * s_el[1][j];
      else L = (T)(a.elen_a[RB->e0 + i] * a.elen_b[CB->e0 + j]);
      for (int c = 0; c < NC; c++) v[c] = L * v[c];
      // pass 0: entry (X, Y) of the block; pass 1: its mirror at (Y, X), with
      // the mirror's own offsets (block assembly places either one anywhere)
      long long X = (pass == 0 ? a.row_off : a.mcol_off) + (long long)a.bpe_a * (RB->e0 + i);
      long long Y = (pass == 0 ? a.col_off : a.mrow_off) + (long long)a.bpe_b * (CB->e0 + j);
      // block entries (dx, dy) -> value
      cx<T> e00 = v[0], e01, e10, e11;
      if (a.bpe_a == 1 && a.bpe_b == 1) {
        if (pass == 0) out[X + Y * ld] = e00; else out[Y + X * ld] = e00;
      } else if (a.bpe_a == 1) {
        e01 = v[1];
        if (pass == 0) { out[X + Y * ld] = e00; out[X + (Y + 1) * ld] = e01; }
        else { out[Y + X * ld] = e00; out[(Y + 1) + X * ld] = e01; }
      } else if (a.bpe_b == 1) {
        e10 = v[1];
        if (pass == 0) { out[X + Y * ld] = e00; out[(X + 1) + Y * ld] = e10; }
        else { out[Y + X * ld] = e00; out[Y + (X + 1) * ld] = e10; }
      } else {
        e01 = v[1]; e10 = v[1]; e11 = v[NC > 2 ? 2 : 0];
        if (pass == 0) {
          out[X + Y * ld] = e00; out[X + 1 + Y * ld] = e10;
          out[X + (Y + 1) * ld] = e01; out[X + 1 + (Y + 1) * ld] = e11;
        } else {
          out[Y + X * ld] = e00; out[Y + 1 + X * ld] = e01;
          out[Y + (X + 1) * ld] = e10; out[Y + 1 + (X + 1) * ld] = e11;
        }
      }
    }
  }
}

static inline cx<double> cxd(double r, double i) { return mk(r, i); }

template <typename T, int NC>
static cudaError_t launch_tiles(const TileArgs& ta, const RegionArgs& ra, int ntiles, cudaStream_t s) {
  size_t smem = (size_t)TE * TE * 4 * NC * sizeof(cx<T>);
  cudaError_t e = cudaFuncSetAttribute(tile_kernel<T, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tile_kernel<T, NC><<<ntiles, 256, smem, s>>>(ta, ra);
  return cudaGetLastError();
}

gbem_status compute_fippi(Geometry* g, cudaStream_t s) {
  for (size_t bi = 0; bi < g->blocks.size(); bi++) {
    DevBlock* db = g->dblocks[bi];
    if (db->nother == 0) continue;
    StatTimer t(ST_NEAR, s);
    fippi_kernel<<<(db->nother + 63) / 64, 64, 0, s>>>(db->near, db->other_list, db->nother, g->d_pv, db->fippi);
    stats_launch(ST_NEAR);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "fippi_kernel");
  }
  g->fippi_ready = true;
  return GBEM_OK;
}

// per-region wavenumbers and PMCHWT/EFIE prefactors of a surface block
// (SurfaceSurfaceInteractions.cc:165-176), signs folded in
static RegionArgs region_args(const Block& b, double wr, double wi, const double* eps, const double* mu) {
  RegionArgs ra;
  memset(&ra, 0, sizeof ra);
  ra.nreg = b.nreg;
  const cx<double> omega = cxd(wr, wi);
  for (int r = 0; r < b.nreg; r++) {
    int R = b.reg[r];
    cx<double> ep = cxd(eps[2 * R], eps[2 * R + 1]), m = cxd(mu[2 * R], mu[2 * R + 1]);
    // k = csqrt2(eps mu) omega, the root with Im >= 0 (libhrutil.cc:692-699)
    cx<double> em = ep * m;
    double rr = std::sqrt(std::hypot(em.re, em.im));
    double th = 0.5 * std::atan2(em.im, em.re);
    cx<double> rt = cxd(rr * std::cos(th), rr * std::sin(th));
    if (rt.im < 0) rt = cxd(-rt.re, -rt.im);
    cx<double> k = rt * omega;
    ra.k[r] = k;
    cx<double> I = cxd(0.0, 1.0);
    double sg = b.sign[r];
    ra.pf1[r] = sg * (I * m * omega);
    cx<double> pf2 = (-sg) * (I * k);
    ra.pfc[r] = (k.re == 0.0 && k.im == 0.0) ? cxd(0.0, 0.0) : cdiv(pf2, I * k);
    ra.pf3[r] = (-sg) * (I * ep * omega);
  }
  return ra;
}

gbem_status assemble_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int precision,
                            void* dM, int ld, int dtype, cudaStream_t s, const BlockSel* only, int only_region) {
  if ((precision == GBEM_PREC_FP64 && dtype != GBEM_C128) || (precision == GBEM_PREC_MIXED && dtype != GBEM_C64)) {
    set_error("gbem_assemble: matrix dtype does not match the precision (C128 for FP64, C64 for MIXED)");
    return GBEM_EINVAL;
  }
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  if (!g->fippi_ready) {
    st = compute_fippi(g, s);
    if (st != GBEM_OK) return st;
  }
  bool any_empty = only_region >= 0;  // a single region leaves blocks without it at zero
  for (const Block& b : g->blocks)
    if (!only || (b.sa == std::min(only->nsa, only->nsb) && b.sb == std::max(only->nsa, only->nsb)))
      any_empty |= (b.nreg == 0);
  size_t esz = dtype == GBEM_C128 ? 16 : 8;
  if (any_empty) {
    // surfaces that share no region interact with zero: clear what is written
    cudaError_t e;
    if (!only) {
      e = cudaMemset2DAsync(dM, (size_t)ld * esz, 0, (size_t)g->N * esz, g->N, s);
    } else {
      const int na = g->S[only->nsa].ne * (g->S[only->nsa].pec ? 1 : 2);
      const int nb = g->S[only->nsb].ne * (g->S[only->nsb].pec ? 1 : 2);
      e = cudaMemset2DAsync((char*)dM + ((size_t)only->row0 + (size_t)only->col0 * ld) * esz, (size_t)ld * esz, 0,
                            (size_t)na * esz, nb, s);
    }
    if (e != cudaSuccess) return cuda_status(e, "memset matrix");
  }
  int* d_status = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_status, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e, "status word");
  for (size_t bi = 0; bi < g->blocks.size(); bi++) {
    const Block& b = g->blocks[bi];
    DevBlock* db = g->dblocks[bi];
    if (b.nreg == 0) continue;
    if (only && !(b.sa == std::min(only->nsa, only->nsb) && b.sb == std::max(only->nsa, only->nsb))) continue;
    RegionArgs ra = region_args(b, wr, wi, eps, mu);
    if (only_region >= 0) {
      // one region's contribution with the sign of an exterior region:
      // KK = i mu w GC0, KN = NK = -i k GC1, NN = -i eps w GC0
      RegionArgs rb;
      memset(&rb, 0, sizeof rb);
      for (int r = 0; r < ra.nreg; r++) {
        if (b.reg[r] != only_region) continue;
        const int R = b.reg[r];
        const cx<double> I = cxd(0.0, 1.0), w = cxd(wr, wi);
        rb.k[0] = ra.k[r];
        rb.pf1[0] = I * cxd(mu[2 * R], mu[2 * R + 1]) * w;
        rb.pfc[0] = cxd(-1.0, 0.0);
        rb.pf3[0] = (-1.0) * (I * cxd(eps[2 * R], eps[2 * R + 1]) * w);
        rb.nreg = 1;
      }
      if (rb.nreg == 0) continue;
      ra = rb;
    }
    {
      StatTimer tn(ST_NEAR, s);
      if (db->nself) {
        stats_launch(ST_NEAR);
        self_kernel<<<(db->nself + 3) / 4, 128, 0, s>>>(db->near, db->self_list, db->nself, g->d_pv, ra, db->nearval);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "self_kernel");
      }
      if (db->nother) {
        stats_launch(ST_NEAR);
        near_kernel<<<(db->nother + 63) / 64, 64, 0, s>>>(db->near, db->other_list, db->nother, g->d_pv, db->fippi,
                                                          ra, db->nearval, d_status);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "near_kernel");
        // touching pairs in the short-wavelength regime (only when some k |r| can exceed pi)
        double kmax = 0.0;
        for (int r = 0; r < b.nreg; r++) kmax = std::fmax(kmax, std::hypot(ra.k[r].re, ra.k[r].im));
        if (kmax * b.rmax_touch > M_PI) {
          stats_launch(ST_NEAR);
          td_touch_kernel<<<(db->nother + 3) / 4, 128, 0, s>>>(db->near, db->other_list, db->nother, g->d_pv, ra,
                                                               db->nearval);
          if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "td_touch_kernel");
        }
      }
    }
    TileArgs ta;
    ta.rows = db->rows; ta.cols = db->cols; ta.tiles = db->tiles;
    ta.pv = g->d_pv; ta.pc = g->d_pc; ta.elen_a = db->elen_a; ta.elen_b = db->elen_b;
    ta.nptr = db->nptr; ta.ncol = db->ncol; ta.nidx = db->nidx; ta.nearval = db->nearval;
    ta.row_panel_offset = g->S[b.sa].panel_offset;
    ta.bpe_a = b.bpe_a; ta.bpe_b = b.bpe_b;
    ta.row_off = g->S[b.sa].bf_offset; ta.col_off = g->S[b.sb].bf_offset;
    ta.mrow_off = ta.col_off; ta.mcol_off = ta.row_off;
    ta.passes = 3;
    if (only) {
      // block assembly: the (nsa, nsb) block at (row0, col0) of dM
      if (b.sa == only->nsa) {
        ta.row_off = only->row0; ta.col_off = only->col0;
        ta.mrow_off = only->row0; ta.mcol_off = only->col0;  // a self block mirrors into itself
        ta.passes = b.sym ? 3 : 1;
      } else {
        ta.mrow_off = only->row0; ta.mcol_off = only->col0;  // (nsa, nsb) is the mirror of (sb, sa)
        ta.passes = 2;
      }
    }
    ta.sym = b.sym ? 1 : 0;
    ta.out = dM; ta.ld = ld;
    int nc = (b.bpe_a == 2 && b.bpe_b == 2) ? 3 : ((b.bpe_a == 1 && b.bpe_b == 1) ? 1 : 2);
    StatTimer tf(ST_FAR, s);
    stats_launch(ST_FAR);
    if (precision == GBEM_PREC_MIXED) {
      e = nc == 1 ? launch_tiles<float, 1>(ta, ra, db->ntiles, s)
                  : nc == 2 ? launch_tiles<float, 2>(ta, ra, db->ntiles, s) : launch_tiles<float, 3>(ta, ra, db->ntiles, s);
    } else {
      e = nc == 1 ? launch_tiles<double, 1>(ta, ra, db->ntiles, s)
                  : nc == 2 ? launch_tiles<double, 2>(ta, ra, db->ntiles, s) : launch_tiles<double, 3>(ta, ra, db->ntiles, s);
    }
    if (e != cudaSuccess) return cuda_status(e, "tile_kernel");
  }
  int h_status = 0;
  e = cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaFreeAsync(d_status, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "assembly");
  if (h_status) {
    set_error("touching panel pairs in the short-wavelength regime (|k r| > pi) need the full-kernel "
              "Taylor-Duffy path, which this build does not implement");
    return GBEM_ENOTSUP;
  }
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// Gradient blocks dM/dx_mu of one surface block (AssembleBEMMatrixBlock with
// GradM, the scuff-cas3D force path): one thread per edge pair, the four
// panel pairs integrated directly with the reference's gradient integrand
// (PanelPanelInteractions.cc:166-181):
//   GradH[2mu]   = int int R_mu hPlus Psi,
//   GradH[2mu+1] = int int (R_mu hTimes Zeta + (F x F')_mu Psi),
// hPlus = F.F' - 4/k^2, hTimes = (F x F').R, Zeta = Phi (-k^2 - 3ik/r + 3/r^2)/r^2.
// Rules as the reference chooses them: far pairs (rRel > 4) the 6x6 rule;
// near pairs the high-order rule without desingularisation; pairs that take
// the Taylor-Duffy branch (ncv = 3, or ncv > 0 when |k r| > pi) contribute
// zero (PanelPanelInteractions.cc:488).  Stamped like GC (GradGC[1] carries
// the 1/(ik) of GC[1]).
// ---------------------------------------------------------------------------
struct GradArgs {
  const double* V;   // vertices of both surfaces' panels: global panel vertex table (9 per panel)
  const double* pc;  // centroid + radius per global panel
  const int* Ea;     // 8 ints per edge of surface a
  const int* Eb;
  const double* La;  // edge lengths
  const double* Lb;
  int nea, neb, poff_a, poff_b;  // edges; first global panel index of each surface
  const double* Va;  // vertex arrays of the two surfaces (for the Q vertices)
  const double* Vb;
  int bpe_a, bpe_b;
  int row0, col0;
  long long ld;
  void* out[3];
};

__device__ void ppi_grad(const double* Pa, const double* Qa, const double* Pb, const double* Qb, cx<double> k,
                         const double* rule, int npts, cx<double>* GH) {
  const double inv4pi = 0.079577471545947667884;
  const cx<double> ik = mk(-k.im, k.re), ik2 = ik * ik, m4 = cdiv(mk(4.0, 0.0), ik2);
  double A[3], B[3], Ap[3], Bp[3];
  for (int c = 0; c < 3; c++) {
    A[c] = Pa[3 + c] - Pa[c]; B[c] = Pa[6 + c] - Pa[c];
    Ap[c] = Pb[3 + c] - Pb[c]; Bp[c] = Pb[6 + c] - Pb[c];
  }
  for (int m = 0; m < 6; m++) GH[m] = mk(0.0, 0.0);
  for (int i = 0; i < npts; i++) {
    const double u = rule[3 * i], v = rule[3 * i + 1], wi = rule[3 * i + 2];
    double x[3], F[3];
    for (int c = 0; c < 3; c++) { x[c] = Pa[c] + u * A[c] + v * B[c]; F[c] = x[c] - Qa[c]; }
    for (int j = 0; j < npts; j++) {
      const double up = rule[3 * j], vp = rule[3 * j + 1], wj = rule[3 * j + 2];
      double xp[3], Fp[3], R[3];
      for (int c = 0; c < 3; c++) {
        xp[c] = Pb[c] + up * Ap[c] + vp * Bp[c];
        Fp[c] = xp[c] - Qb[c];
        R[c] = x[c] - xp[c];
      }
      const double r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2], r = sqrt(r2), ri = 1.0 / r;
      double sn, cs;
      sincos(k.re * r, &sn, &cs);
      const double amp = wi * wj * inv4pi * ri * exp(-k.im * r);
      const cx<double> Phi = mk(amp * cs, amp * sn);
      const cx<double> Psi = Phi * mk(ik.re - ri, ik.im) * mk(ri, 0.0);
      const cx<double> Zeta = Phi * (ik2 - mk(3.0 * ri, 0.0) * ik + mk(3.0 * ri * ri, 0.0)) * mk(ri * ri, 0.0);
      const cx<double> hPlus = mk(F[0] * Fp[0] + F[1] * Fp[1] + F[2] * Fp[2], 0.0) + m4;
      double X[3];
      vcross(F, Fp, X);
      const double hT = X[0] * R[0] + X[1] * R[1] + X[2] * R[2];
      const cx<double> hPsi = hPlus * Psi;
      const cx<double> hZ = hT * Zeta;
      for (int mu = 0; mu < 3; mu++) {
        GH[2 * mu] = GH[2 * mu] + R[mu] * hPsi;
        GH[2 * mu + 1] = GH[2 * mu + 1] + R[mu] * hZ + X[mu] * Psi;
      }
    }
  }
}

template <bool REAL>
__global__ void __launch_bounds__(128) grad_kernel(GradArgs a, RegionArgs ra) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.nea * a.neb) return;
  const int ea = (int)(t % a.nea), eb = (int)(t / a.nea);
  const int* EA = a.Ea + 8 * ea;
  const int* EB = a.Eb + 8 * eb;
  const double La = a.La[ea], Lb = a.Lb[eb];
  cx<double> acc[3][4];
  for (int mu = 0; mu < 3; mu++)
    for (int c = 0; c < 4; c++) acc[mu][c] = mk(0.0, 0.0);
  for (int r = 0; r < ra.nreg; r++) {
    const cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    cx<double> S0[3], S1[3];
    for (int mu = 0; mu < 3; mu++) { S0[mu] = mk(0.0, 0.0); S1[mu] = mk(0.0, 0.0); }
    for (int sa = 0; sa < 2; sa++) {
      const int iqa = sa == 0 ? EA[2] : EA[3];
      const int pa = sa == 0 ? EA[4] : EA[5];
      if (iqa < 0 || pa < 0) continue;
      for (int sb = 0; sb < 2; sb++) {
        const int iqb = sb == 0 ? EB[2] : EB[3];
        const int pb = sb == 0 ? EB[4] : EB[5];
        if (iqb < 0 || pb < 0) continue;
        const int gpa = a.poff_a + pa, gpb = a.poff_b + pb;
        const double* Pa = a.V + 9 * (size_t)gpa;
        const double* Pb = a.V + 9 * (size_t)gpb;
        const double* ca = a.pc + 4 * (size_t)gpa;
        const double* cb = a.pc + 4 * (size_t)gpb;
        const double rmax = fmax(ca[3], cb[3]);
        const double dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
        const bool far = sqrt(dx * dx + dy * dy + dz * dz) > 4.0 * rmax;
        cx<double> GH[6];
        if (far) {
          ppi_grad(Pa, a.Va + 3 * iqa, Pb, a.Vb + 3 * iqb, k, c_lo64, 6, GH);
        } else {
          int ncv = 0;
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
              const double ex = Pa[3 * i] - Pb[3 * j], ey = Pa[3 * i + 1] - Pb[3 * j + 1], ez = Pa[3 * i + 2] - Pb[3 * j + 2];
              if (sqrt(ex * ex + ey * ey + ez * ez) < 1e-6 * rmax) ncv++;
            }
          const bool swr = hypot(k.re * rmax, k.im * rmax) > M_PI;
          if (ncv == 3 || (ncv > 0 && swr)) continue;  // Taylor-Duffy pairs: zero gradient
          ppi_grad(Pa, a.Va + 3 * iqa, Pb, a.Vb + 3 * iqb, k, c_ho, HO_N * HO_N, GH);
        }
        const double sg = (sa == sb) ? 1.0 : -1.0;
        for (int mu = 0; mu < 3; mu++) {
          S0[mu] = S0[mu] + sg * GH[2 * mu];
          S1[mu] = S1[mu] + sg * GH[2 * mu + 1];
        }
      }
    }
    const double LL = La * Lb;
    for (int mu = 0; mu < 3; mu++) {
      const cx<double> g0 = LL * S0[mu], g1 = LL * S1[mu];
      acc[mu][0] = acc[mu][0] + ra.pf1[r] * g0;
      acc[mu][1] = acc[mu][1] + ra.pfc[r] * g1;
      acc[mu][3] = acc[mu][3] + ra.pf3[r] * g0;
    }
  }
  const long long X = a.row0 + (long long)a.bpe_a * ea, Y = a.col0 + (long long)a.bpe_b * eb;
  for (int mu = 0; mu < 3; mu++) {
    if (!a.out[mu]) continue;
    // (K,K) = PF1 G0; (K,N) = (N,K) = PF2 G1 / (ik); (N,N) = PF3 G0
    cx<double> e[2][2] = {{acc[mu][0], acc[mu][1]}, {acc[mu][1], acc[mu][3]}};
    for (int dx = 0; dx < a.bpe_a; dx++)
      for (int dy = 0; dy < a.bpe_b; dy++) {
        const long long idx = (X + dx) + (Y + dy) * a.ld;
        if (REAL) ((double*)a.out[mu])[idx] = e[dx][dy].re;
        else ((cx<double>*)a.out[mu])[idx] = e[dx][dy];
      }
  }
}

gbem_status assemble_gradient_device(Geometry* g, double wr, double wi, const double* eps, const double* mu,
                                     const BlockSel& sel, void* const out[3], int ld, int dtype, cudaStream_t s) {
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  const int lo = std::min(sel.nsa, sel.nsb), hi = std::max(sel.nsa, sel.nsb);
  const Block* bp = nullptr;
  for (const Block& b : g->blocks)
    if (b.sa == lo && b.sb == hi) bp = &b;
  if (!bp) { set_error("gradient: no such surface block"); return GBEM_EINVAL; }
  const Surface& A = g->S[sel.nsa];
  const Surface& B = g->S[sel.nsb];
  const size_t es = dtype == GBEM_F64 ? 8 : 16;
  cudaError_t e = cudaSuccess;
  // the block's entries are written by one thread each; a block of surfaces
  // that share no region is zero
  for (int m = 0; m < 3 && e == cudaSuccess; m++)
    if (out[m])
      e = cudaMemset2DAsync((char*)out[m] + ((size_t)sel.row0 + (size_t)sel.col0 * ld) * es, (size_t)ld * es, 0,
                            (size_t)A.ne * (A.pec ? 1 : 2) * es, B.ne * (B.pec ? 1 : 2), s);
  if (e != cudaSuccess) return cuda_status(e, "gradient memset");
  if (bp->nreg == 0 || A.ne == 0 || B.ne == 0) return GBEM_OK;
  double *dVa = nullptr, *dVb = nullptr, *dLa = nullptr, *dLb = nullptr;
  int *dEa = nullptr, *dEb = nullptr;
  e = dupload(&dVa, A.V.data(), A.V.size());
  if (e == cudaSuccess) e = dupload(&dVb, B.V.data(), B.V.size());
  if (e == cudaSuccess) e = dupload(&dEa, A.E.data(), A.E.size());
  if (e == cudaSuccess) e = dupload(&dEb, B.E.data(), B.E.size());
  if (e == cudaSuccess) e = dupload(&dLa, A.elen.data(), A.elen.size());
  if (e == cudaSuccess) e = dupload(&dLb, B.elen.data(), B.elen.size());
  if (e == cudaSuccess) {
    GradArgs ga;
    ga.V = g->d_pv; ga.pc = g->d_pc; ga.Ea = dEa; ga.Eb = dEb; ga.La = dLa; ga.Lb = dLb;
    ga.nea = A.ne; ga.neb = B.ne; ga.poff_a = A.panel_offset; ga.poff_b = B.panel_offset;
    ga.Va = dVa; ga.Vb = dVb;
    ga.bpe_a = A.pec ? 1 : 2; ga.bpe_b = B.pec ? 1 : 2;
    ga.row0 = sel.row0; ga.col0 = sel.col0; ga.ld = ld;
    for (int m = 0; m < 3; m++) ga.out[m] = out[m];
    const RegionArgs ra = region_args(*bp, wr, wi, eps, mu);
    const long long n = (long long)A.ne * B.ne;
    stats_launch(ST_OTHER);
    if (dtype == GBEM_F64) grad_kernel<true><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(ga, ra);
    else grad_kernel<false><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(ga, ra);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFree(dVa); cudaFree(dVb); cudaFree(dEa); cudaFree(dEb); cudaFree(dLa); cudaFree(dLb);
  return cuda_status(e, "gradient block");
}

// ---------------------------------------------------------------------------
// plane-wave right-hand side (AssembleRHSVector.cc:145-255, 288-340 with a
// PlaneWave source in the exterior region, libs/libIncField/PlaneWave.cc:71-87)
//   K entry: -<f_n, E_inc>/ZVAC,  N entry: -<f_n, H_inc>  (dielectric surfaces)
// ---------------------------------------------------------------------------
struct RhsArgs {
  const double* V;  // surface vertices
  const int* E;     // 8 ints per edge
  const double* elen;
  int ne, bf_offset, pec, sign;  // sign: -1 incident field outside, +1 inside
  cx<double> k, Z;               // wavenumber and wave impedance of the source region
  cx<double> E0[3];
  double nh[3];
  cx<double>* rhs;
};

__device__ void pw_fields(const RhsArgs& a, const double* X, cx<double>* Ef, cx<double>* Hf) {
  double ph = a.nh[0] * X[0] + a.nh[1] * X[1] + a.nh[2] * X[2];
  cx<double> ex = cexpo(mk(-a.k.im * ph, a.k.re * ph));
  for (int i = 0; i < 3; i++) Ef[i] = a.E0[i] * ex;
  Hf[0] = cdiv(a.nh[1] * Ef[2] - a.nh[2] * Ef[1], a.Z);
  Hf[1] = cdiv(a.nh[2] * Ef[0] - a.nh[0] * Ef[2], a.Z);
  Hf[2] = cdiv(a.nh[0] * Ef[1] - a.nh[1] * Ef[0], a.Z);
}

__global__ void rhs_kernel(RhsArgs a) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne) return;
  const int* ed = a.E + 8 * e;
  const double* V1 = a.V + 3 * ed[0];
  const double* V2 = a.V + 3 * ed[1];
  cx<double> Ep = mk(0.0, 0.0), Hp = mk(0.0, 0.0);
  for (int side = 0; side < 2; side++) {
    int iq = side == 0 ? ed[2] : ed[3];
    if (iq < 0) continue;
    const double* Q = a.V + 3 * iq;
    double A[3], B[3];
    for (int i = 0; i < 3; i++) { A[i] = V1[i] - Q[i]; B[i] = V2[i] - Q[i]; }
    cx<double> se = mk(0.0, 0.0), sh = mk(0.0, 0.0);
    for (int q = 0; q < HO_N * HO_N; q++) {
      double u = c_ho[3 * q], v = c_ho[3 * q + 1], w = c_ho[3 * q + 2];
      double X[3], F[3];
      for (int i = 0; i < 3; i++) { F[i] = u * A[i] + v * B[i]; X[i] = Q[i] + F[i]; }
      cx<double> Ef[3], Hf[3];
      pw_fields(a, X, Ef, Hf);
      for (int i = 0; i < 3; i++) { se = se + (w * F[i]) * Ef[i]; sh = sh + (w * F[i]) * Hf[i]; }
    }
    // (L/2A) int (X-Q).E dA = L int_std (X-Q).E
    double L = a.elen[e];
    if (side == 0) { Ep = Ep + L * se; Hp = Hp + L * sh; }
    else { Ep = Ep - L * se; Hp = Hp - L * sh; }
  }
  const double ZVAC = 376.73031346177;
  double sg = (double)a.sign;
  if (a.pec) a.rhs[a.bf_offset + e] = (sg / ZVAC) * Ep;
  else {
    a.rhs[a.bf_offset + 2 * e] = (sg / ZVAC) * Ep;
    a.rhs[a.bf_offset + 2 * e + 1] = sg * Hp;
  }
}

gbem_status rhs_planewave_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, const double* E0,
                                 const double* nh, void* d_rhs, cudaStream_t s) {
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  cudaError_t e = cudaMemsetAsync(d_rhs, 0, sizeof(double) * 2 * g->N, s);
  if (e != cudaSuccess) return cuda_status(e, "rhs memset");
  for (Surface& S : g->S) {
    // the incident field lives in region 0 (the exterior medium)
    int sign;
    if (S.reg_ext == 0) sign = -1;
    else if (S.reg_int == 0) sign = 1;
    else continue;
    RhsArgs a;
    double *dV = nullptr, *dL = nullptr;
    int* dE = nullptr;
    e = dupload(&dV, S.V.data(), S.V.size());
    if (e == cudaSuccess) e = dupload(&dE, S.E.data(), S.E.size());
    if (e == cudaSuccess) e = dupload(&dL, S.elen.data(), S.elen.size());
    if (e != cudaSuccess) return cuda_status(e, "rhs upload");
    a.V = dV; a.E = dE; a.elen = dL; a.ne = S.ne; a.bf_offset = S.bf_offset; a.pec = S.pec ? 1 : 0; a.sign = sign;
    cx<double> ep = cxd(eps[0], eps[1]), m = cxd(mu[0], mu[1]), em = ep * m;
    double rr = std::sqrt(std::hypot(em.re, em.im)), th = 0.5 * std::atan2(em.im, em.re);
    cx<double> rt = cxd(rr * std::cos(th), rr * std::sin(th));  // principal sqrt, as std::sqrt
    a.k = rt * cxd(wr, wi);
    cx<double> q = cdiv(m, ep);
    double rq = std::sqrt(std::hypot(q.re, q.im)), tq = 0.5 * std::atan2(q.im, q.re);
    a.Z = 376.73031346177 * cxd(rq * std::cos(tq), rq * std::sin(tq));
    for (int i = 0; i < 3; i++) { a.E0[i] = cxd(E0[2 * i], E0[2 * i + 1]); a.nh[i] = nh[i]; }
    a.rhs = (cx<double>*)d_rhs;
    if (S.ne) rhs_kernel<<<(S.ne + 127) / 128, 128, 0, s>>>(a);
    e = cudaGetLastError();
    cudaStreamSynchronize(s);
    cudaFree(dV); cudaFree(dE); cudaFree(dL);
    if (e != cudaSuccess) return cuda_status(e, "rhs_kernel");
  }
  return GBEM_OK;
}

}  // namespace gbem
